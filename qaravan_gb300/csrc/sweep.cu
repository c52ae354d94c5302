// Fused sweep: several gates per read+write of the state.
//
// The reference applies every gate as a separate contraction over the whole
// state (core/base_sim.py:30-53 -> tensorQ/statevector_sim.py:124-140). Here
// the host compiler groups consecutive gates whose qubits fit one tile: a CTA
// stages a tile of 2^m amplitudes -- the low `L` flat bits (contiguous runs of
// 2^L amplitudes) times every combination of `H` chosen high bits -- in
// shared memory, applies the whole op list to it, and writes it back. HBM
// traffic is one read and one write of the state per sweep instead of per
// gate.
//
// Two kernels share the in-tile math (sweep_common.cuh):
//  * sweep_ldst_kernel (here), the default: every thread issues 16-byte
//    cp.async copies of the next tile into a second buffer while the ops run
//    on the current one, and writes results back with 16-byte stores;
//  * sweep_tma_kernel (sweep_tma.cu), selected with qgb_set_sweep_impl(1) or
//    QGB_SWEEP_IMPL=tma: TMA tensor copies with the hardware 128-byte swizzle
//    into a ring of buffers, fed by a dedicated producer warp. On the 28-qubit
//    brickwork it measured slower than the cp.async kernel (its 256-byte
//    boxes are too small for the copy engine), so it is not the default.
#include <cstdlib>
#include <cstring>

#include "sweep_common.cuh"

namespace qgb {

constexpr int kLdstMaxThreads = 512;

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(uint32_t(__cvta_generic_to_shared(smem_dst))),
                 "l"(gmem_src)
                 : "memory");
}

// nbuf = 2: the copy of tile i+1 (cp.async, 16 bytes per thread-instruction,
// no register staging) is in flight while the ops run on tile i.
template <typename T, int KMAX>
__global__ void __launch_bounds__(kLdstMaxThreads) sweep_ldst_kernel(cplx<T>* __restrict__ sv,
                                                                     const cplx<T>* __restrict__ mats,
                                                                     const __grid_constant__ SweepArgs a, int nbuf) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = a.sw.low_bits, H = a.sw.n_high, m = L + H;
    // layout: nbuf tiles (2^m complex each) | matrix stage | hoff (2^H uint64); complex regions 16-byte aligned
    C* bufs = reinterpret_cast<C*>(smem_raw);
    C* msh = bufs + (size_t(nbuf) << m);
    uint64_t* hoff = reinterpret_cast<uint64_t*>(msh + stage_elems<KMAX>());
    for (uint32_t h = threadIdx.x; h < (1u << H); h += blockDim.x) {
        uint64_t o = 0;
        for (int j = 0; j < H; ++j) o |= uint64_t((h >> j) & 1u) << a.sw.high_bits[j];
        hoff[h] = o;
    }
    __syncthreads();
    const uint32_t lmask = (1u << L) - 1;
    constexpr uint32_t per16 = 16 / sizeof(C);  // amplitudes per 16-byte copy
    const uint64_t total = uint64_t(a.batch) * a.tiles;
    auto base_of = [&](uint64_t w) -> uint64_t {
        const uint64_t b = w / a.tiles, o = w - b * a.tiles;
        uint64_t base = uint64_t(b) * uint64_t(a.sv_stride);
        for (int j = 0; j < a.n_outer; ++j) base |= ((o >> j) & 1ull) << a.outer_bits[j];
        return base;  // batch offset plus the scattered tile index (disjoint bits)
    };
    auto load_async = [&](uint64_t w, C* dst) {
        const uint64_t base = base_of(w);
        for (uint32_t e = per16 * threadIdx.x; e < (1u << m); e += per16 * blockDim.x)
            cp_async16(dst + swz<T>(e), sv + (base + (hoff[e >> L] | (e & lmask))));
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    uint64_t w = blockIdx.x;
    if (w < total) load_async(w, bufs);
    for (uint32_t i = 0; w < total; ++i, w += gridDim.x) {
        C* cur = bufs + (size_t(nbuf == 2 ? (i & 1) : 0) << m);
        const uint64_t wn = w + gridDim.x;
        if (nbuf == 2 && wn < total) {
            load_async(wn, bufs + (size_t((i + 1) & 1) << m));
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        apply_ops<T, KMAX, CtaSync>(cur, m, a, mats + int64_t(w / a.tiles) * a.mat_stride, msh, threadIdx.x,
                                    blockDim.x);
        const uint64_t base = base_of(w);
        for (uint32_t e = per16 * threadIdx.x; e < (1u << m); e += per16 * blockDim.x)
            *reinterpret_cast<float4*>(sv + (base + (hoff[e >> L] | (e & lmask)))) =
                *reinterpret_cast<const float4*>(cur + swz<T>(e));
        __syncthreads();  // the buffer is free for the copy issued two tiles later
        if (nbuf == 1 && wn < total) load_async(wn, bufs);
    }
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

namespace {

template <typename T>
size_t ldst_smem_bytes(int m, int H, int kmax_inst, int nbuf) {
    size_t stage = kmax_inst >= 3 ? (size_t(1) << (2 * (kmax_inst < kStageK ? kmax_inst : kStageK))) : 0;
    return sizeof(cplx<T>) * ((size_t(nbuf) << m) + stage) + sizeof(uint64_t) * (size_t(1) << H);
}

template <typename T, int KMAX>
int launch_ldst(void* sv, const void* mats, const SweepArgs& a, cudaStream_t st) {
    const int m = a.sw.low_bits + a.sw.n_high;
    auto kern = sweep_ldst_kernel<T, KMAX>;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
            return check_launch("sweep attribute");
        attr = true;
    }
    // prefer a double buffer; when a single CTA fits per SM give it 512 threads
    for (int nbuf = 2; nbuf >= 1; --nbuf) {
        const size_t smem = ldst_smem_bytes<T>(m, a.sw.n_high, KMAX, nbuf);
        if (smem > 227 * 1024) continue;
        int per_sm = 0, threads = 256;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem) != cudaSuccess)
            return check_launch("sweep occupancy");
        if (per_sm < 1) continue;
        if (per_sm == 1) {
            int p512 = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p512, kern, 512, smem) != cudaSuccess)
                return check_launch("sweep occupancy");
            if (p512 >= 1) threads = 512;
        }
        const uint64_t total = uint64_t(a.batch) * a.tiles;
        uint64_t grid = uint64_t(per_sm) * sm_count();
        if (grid > total) grid = total;
        kern<<<unsigned(grid), threads, smem, st>>>((cplx<T>*)sv, (const cplx<T>*)mats, a, nbuf);
        return check_launch("sweep kernel");
    }
    return set_error(QGB_EINVAL, "sweep tile of 2^%d amplitudes does not fit in shared memory", m);
}

template <typename T>
int dispatch_ldst(void* sv, const void* mats, const SweepArgs& a, int kmax, cudaStream_t st) {
    switch (kmax) {
        case 1:
        case 2: return launch_ldst<T, 2>(sv, mats, a, st);
        case 3: return launch_ldst<T, 3>(sv, mats, a, st);
        case 4: return launch_ldst<T, 4>(sv, mats, a, st);
        case 5:
            if constexpr (sizeof(T) == 4) return launch_ldst<T, 5>(sv, mats, a, st);
    }
    return set_error(QGB_EINVAL, "sweep op width %d unsupported for this dtype", kmax);
}

int g_sweep_impl = -1;  // 0 = cp.async load/store kernel, 1 = TMA kernel when eligible

int sweep_impl() {
    if (g_sweep_impl < 0) {
        const char* e = getenv("QGB_SWEEP_IMPL");
        g_sweep_impl = (e && strcmp(e, "tma") == 0) ? 1 : 0;
    }
    return g_sweep_impl;
}

}  // namespace

extern "C" int qgb_set_sweep_impl(int impl) {
    if (impl != 0 && impl != 1) return set_error(QGB_EINVAL, "sweep implementation %d unknown (0 = load/store, 1 = TMA)", impl);
    g_sweep_impl = impl;
    return QGB_OK;
}

extern "C" int qgb_apply_sweep(void* sv, int dtype, int n, const qgb_sweep* sweep, const void* mats,
                               int64_t mat_stride, int64_t batch, int64_t sv_stride, void* stream) {
    if (!sv || !sweep || (!mats && sweep->n_ops > 0)) return set_error(QGB_EINVAL, "null pointer");
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    if (n < 1 || n > 2 * QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid", n);
    if (batch < 1) return set_error(QGB_EINVAL, "batch %lld < 1", (long long)batch);
    if (batch > 1 && sv_stride < (int64_t(1) << n)) return set_error(QGB_EINVAL, "state stride too small");
    if (mat_stride < 0 || (mat_stride & 1)) return set_error(QGB_EINVAL, "matrix stride must be even and non-negative");
    const size_t esz = dtype == QGB_C64 ? 8 : 16;
    if ((reinterpret_cast<uintptr_t>(sv) & 15) || (batch > 1 && (sv_stride * int64_t(esz)) % 16))
        return set_error(QGB_EINVAL, "state pointer and stride must be 16-byte aligned");
    if (mats && (reinterpret_cast<uintptr_t>(mats) % esz)) return set_error(QGB_EINVAL, "matrix buffer misaligned");
    const qgb_sweep& sw = *sweep;
    const int L = sw.low_bits, H = sw.n_high, m = L + H;
    if (L < 1 || H < 0 || H > QGB_SWEEP_MAX_HIGH || m > n || m > QGB_SWEEP_MAX_TILE_BITS)
        return set_error(QGB_EINVAL, "tile geometry L=%d H=%d invalid for n=%d", L, H, n);
    if (sw.n_ops < 0 || sw.n_ops > QGB_SWEEP_MAX_OPS) return set_error(QGB_EINVAL, "n_ops=%d out of range", sw.n_ops);
    SweepArgs a{};
    a.sw = sw;
    a.n = n;
    uint64_t in_tile = (1ull << L) - 1;
    int prev = L - 1;
    for (int h = 0; h < H; ++h) {
        const int b = sw.high_bits[h];
        if (b <= prev || b >= n) return set_error(QGB_EINVAL, "high bits must be ascending, >= L and < n");
        in_tile |= 1ull << b;
        prev = b;
    }
    a.n_outer = 0;
    for (int b = 0; b < n; ++b)
        if (!((in_tile >> b) & 1ull)) a.outer_bits[a.n_outer++] = b;
    int kmax = 1;
    const int kcap = dtype == QGB_C64 ? 5 : 4;
    for (int i = 0; i < sw.n_ops; ++i) {
        const int k = sw.op_k[i];
        if (k < 1 || k > kcap) return set_error(QGB_EINVAL, "sweep op %d has width %d (max %d)", i, k, kcap);
        if (k > m) return set_error(QGB_EINVAL, "sweep op %d wider than the tile", i);
        uint32_t seen = 0;
        for (int j = 0; j < k; ++j) {
            const int p = sw.op_pos[i][j];
            if (p < 0 || p >= m || ((seen >> p) & 1u)) return set_error(QGB_EINVAL, "sweep op %d has bad tile bit %d", i, p);
            seen |= 1u << p;
        }
        if (sw.op_mat[i] < 0) return set_error(QGB_EINVAL, "sweep op %d has negative matrix offset", i);
        if (dtype == QGB_C64 && k >= 3 && (sw.op_mat[i] & 1))
            return set_error(QGB_EINVAL, "sweep op %d: complex64 matrices of width >= 3 need an even (16-byte) offset", i);
        if (k > kmax) kmax = k;
    }
    a.mat_stride = mat_stride;
    a.batch = batch;
    a.sv_stride = sv_stride;
    a.tiles = uint64_t(1) << (n - m);
    cudaStream_t st = (cudaStream_t)stream;
    if (sweep_impl() == 1) {
        const int rc = launch_sweep_tma(dtype, sv, mats, a, kmax, st);
        if (rc != 1) return rc;
    }
    if (dtype == QGB_C128 && c128_arith() == 1) return launch_sweep_df(sv, mats, a, kmax, st);
    return dtype == QGB_C64 ? dispatch_ldst<float>(sv, mats, a, kmax, st) : dispatch_ldst<double>(sv, mats, a, kmax, st);
}
