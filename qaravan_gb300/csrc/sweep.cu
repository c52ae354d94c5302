// Fused sweep: several gates per read+write of the state.
//
// The reference applies every gate as a separate contraction over the whole
// state (core/base_sim.py:30-53 -> tensorQ/statevector_sim.py:124-140). Here
// the host compiler groups consecutive gates whose qubits fit one tile: a CTA
// stages a tile of 2^m amplitudes -- the low `L` flat bits (contiguous runs of
// 2^L amplitudes, coalesced 16-byte loads) times every combination of `H`
// chosen high bits -- in shared memory, applies the whole op list to it, and
// writes it back. HBM traffic is one read and one write of the state per
// sweep instead of per gate; the op math runs out of shared memory (swizzled
// on 16-byte granules against bank conflicts) with the small matrices in
// registers.
#include "qgb_common.cuh"

namespace qgb {

struct SweepArgs {
    qgb_sweep sw;
    int n;  // bits per vector
    int n_outer;
    int outer_bits[2 * QGB_MAX_QUBITS];
    int64_t mat_stride, batch, sv_stride;
    uint64_t tiles;  // tiles per vector
};

constexpr int kSweepThreads = 256;
constexpr int kStageK = 4;  // ops with k >= 3 stage their matrix in shared memory (k <= 4)

template <typename T, int K>
__device__ __forceinline__ void tile_op(cplx<T>* __restrict__ tile, int m, const int* pos_in,
                                        const cplx<T>* __restrict__ mat, cplx<T>* __restrict__ msh) {
    constexpr int D = 1 << K;
    using C = cplx<T>;
    int pos[K], srt[K];
#pragma unroll
    for (int j = 0; j < K; ++j) pos[j] = srt[j] = pos_in[j];
#pragma unroll
    for (int i = 1; i < K; ++i)
#pragma unroll
        for (int j = i; j > 0; --j)
            if (srt[j - 1] > srt[j]) {
                int t = srt[j];
                srt[j] = srt[j - 1];
                srt[j - 1] = t;
            }
    uint32_t off[D];
#pragma unroll
    for (int r = 0; r < D; ++r) {
        uint32_t o = 0;
#pragma unroll
        for (int j = 0; j < K; ++j) o |= uint32_t((r >> (K - 1 - j)) & 1) << pos[j];
        off[r] = o;
    }
    const uint32_t groups = 1u << (m - K);
    if constexpr (K <= 2) {
        C mr[D * D];
#pragma unroll
        for (int i = 0; i < D * D; ++i) mr[i] = __ldg(&mat[i]);
        for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
            uint32_t base = g;
#pragma unroll
            for (int j = 0; j < K; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
            C v[D];
#pragma unroll
            for (int c = 0; c < D; ++c) v[c] = tile[swz<T>(base | off[c])];
#pragma unroll
            for (int r = 0; r < D; ++r) {
                C acc = mk<T>(0, 0);
#pragma unroll
                for (int c = 0; c < D; ++c) cfma(acc, mr[r * D + c], v[c]);
                tile[swz<T>(base | off[r])] = acc;
            }
        }
    } else {
        const C* mm = mat;
        if constexpr (K <= kStageK) {
            for (int i = threadIdx.x; i < D * D; i += blockDim.x) msh[i] = mat[i];
            __syncthreads();
            mm = msh;
        }
        for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
            uint32_t base = g;
#pragma unroll
            for (int j = 0; j < K; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
            C v[D];
#pragma unroll
            for (int c = 0; c < D; ++c) v[c] = tile[swz<T>(base | off[c])];
#pragma unroll 1
            for (int r = 0; r < D; ++r) {
                const C* mrow = mm + r * D;
                C acc = mk<T>(0, 0);
#pragma unroll
                for (int c = 0; c < D; ++c) cfma(acc, mrow[c], v[c]);
                uint32_t o = 0;
#pragma unroll
                for (int j = 0; j < K; ++j) o |= uint32_t((r >> (K - 1 - j)) & 1) << pos[j];
                tile[swz<T>(base | o)] = acc;
            }
        }
    }
}

template <typename T, int KMAX>
__global__ void __launch_bounds__(kSweepThreads) sweep_kernel(cplx<T>* __restrict__ sv, const cplx<T>* __restrict__ mats,
                                                              const __grid_constant__ SweepArgs a) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = a.sw.low_bits, H = a.sw.n_high, m = L + H;
    // layout: tile (2^m complex) | matrix stage (4^min(KMAX,4) complex) | hoff (2^H uint64);
    // both complex regions start on 16-byte boundaries
    C* tile = reinterpret_cast<C*>(smem_raw);
    C* msh = tile + (1u << m);
    constexpr int kStage = KMAX >= 3 ? (1 << (2 * (KMAX < kStageK ? KMAX : kStageK))) : 0;
    uint64_t* hoff = reinterpret_cast<uint64_t*>(msh + kStage);
    for (uint32_t h = threadIdx.x; h < (1u << H); h += blockDim.x) {
        uint64_t o = 0;
        for (int j = 0; j < H; ++j) o |= uint64_t((h >> j) & 1u) << a.sw.high_bits[j];
        hoff[h] = o;
    }
    const uint32_t lmask = (1u << L) - 1;
    const uint64_t total = uint64_t(a.batch) * a.tiles;
    for (uint64_t w = blockIdx.x; w < total; w += gridDim.x) {
        const uint64_t b = w / a.tiles, o = w - b * a.tiles;
        C* s = sv + int64_t(b) * a.sv_stride;
        const C* mb = mats + int64_t(b) * a.mat_stride;
        uint64_t base = 0;
        for (int j = 0; j < a.n_outer; ++j) base |= ((o >> j) & 1ull) << a.outer_bits[j];
        __syncthreads();  // hoff ready; previous tile fully stored
        if constexpr (sizeof(T) == 4) {
            for (uint32_t e = 2 * threadIdx.x; e < (1u << m); e += 2 * blockDim.x) {
                const uint64_t gi = base | hoff[e >> L] | (e & lmask);
                const float4 v = *reinterpret_cast<const float4*>(s + gi);
                *reinterpret_cast<float4*>(tile + swz<T>(e)) = v;
            }
        } else {
            for (uint32_t e = threadIdx.x; e < (1u << m); e += blockDim.x) {
                const uint64_t gi = base | hoff[e >> L] | (e & lmask);
                tile[swz<T>(e)] = s[gi];
            }
        }
        __syncthreads();
        for (int i = 0; i < a.sw.n_ops; ++i) {
            const int k = a.sw.op_k[i];
            const C* mat = mb + a.sw.op_mat[i];
            const int* pos = a.sw.op_pos[i];
            if (k == 1) tile_op<T, 1>(tile, m, pos, mat, msh);
            else if (k == 2) { if constexpr (KMAX >= 2) tile_op<T, 2>(tile, m, pos, mat, msh); }
            else if (k == 3) { if constexpr (KMAX >= 3) tile_op<T, 3>(tile, m, pos, mat, msh); }
            else if (k == 4) { if constexpr (KMAX >= 4) tile_op<T, 4>(tile, m, pos, mat, msh); }
            else if (k == 5) { if constexpr (KMAX >= 5) tile_op<T, 5>(tile, m, pos, mat, msh); }
            __syncthreads();
        }
        if constexpr (sizeof(T) == 4) {
            for (uint32_t e = 2 * threadIdx.x; e < (1u << m); e += 2 * blockDim.x) {
                const uint64_t gi = base | hoff[e >> L] | (e & lmask);
                *reinterpret_cast<float4*>(s + gi) = *reinterpret_cast<const float4*>(tile + swz<T>(e));
            }
        } else {
            for (uint32_t e = threadIdx.x; e < (1u << m); e += blockDim.x) {
                const uint64_t gi = base | hoff[e >> L] | (e & lmask);
                s[gi] = tile[swz<T>(e)];
            }
        }
    }
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

namespace {

template <typename T> constexpr int max_sweep_k() { return sizeof(T) == 4 ? 5 : 4; }

template <typename T>
size_t sweep_smem_bytes(int m, int H, int kmax) {
    // kmax is rounded up to the launched instantiation (1 -> 2)
    if (kmax < 2) kmax = 2;
    size_t stage = kmax >= 3 ? (size_t(1) << (2 * (kmax < kStageK ? kmax : kStageK))) : 0;
    return sizeof(cplx<T>) * ((size_t(1) << m) + stage) + sizeof(uint64_t) * (size_t(1) << H);
}

template <typename T, int KMAX>
int launch_sweep(void* sv, const void* mats, const SweepArgs& a, size_t smem, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(sweep_kernel<T, KMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
            cudaSuccess)
            return check_launch("sweep attribute");
        attr = true;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_kernel<T, KMAX>, kSweepThreads, smem) !=
        cudaSuccess)
        return check_launch("sweep occupancy");
    if (per_sm < 1) return set_error(QGB_EINVAL, "sweep tile of %zu bytes does not fit on an SM", smem);
    const uint64_t total = uint64_t(a.batch) * a.tiles;
    uint64_t grid = uint64_t(per_sm) * sm_count();
    if (grid > total) grid = total;
    sweep_kernel<T, KMAX><<<unsigned(grid), kSweepThreads, smem, st>>>((cplx<T>*)sv, (const cplx<T>*)mats, a);
    return check_launch("sweep kernel");
}

template <typename T>
int dispatch_sweep(void* sv, const void* mats, const SweepArgs& a, int kmax, cudaStream_t st) {
    const int m = a.sw.low_bits + a.sw.n_high;
    const size_t smem = sweep_smem_bytes<T>(m, a.sw.n_high, kmax);
    if (smem > 227 * 1024) return set_error(QGB_EINVAL, "sweep needs %zu bytes of shared memory", smem);
    switch (kmax) {
        case 1:
        case 2: return launch_sweep<T, 2>(sv, mats, a, smem, st);
        case 3: return launch_sweep<T, 3>(sv, mats, a, smem, st);
        case 4: return launch_sweep<T, 4>(sv, mats, a, smem, st);
        case 5:
            if constexpr (max_sweep_k<T>() >= 5) return launch_sweep<T, 5>(sv, mats, a, smem, st);
    }
    return set_error(QGB_EINVAL, "sweep op width %d unsupported for this dtype", kmax);
}

}  // namespace

extern "C" int qgb_apply_sweep(void* sv, int dtype, int n, const qgb_sweep* sweep, const void* mats,
                               int64_t mat_stride, int64_t batch, int64_t sv_stride, void* stream) {
    if (!sv || !sweep || (!mats && sweep->n_ops > 0)) return set_error(QGB_EINVAL, "null pointer");
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    if (n < 1 || n > 2 * QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid", n);
    if (batch < 1) return set_error(QGB_EINVAL, "batch %lld < 1", (long long)batch);
    if (batch > 1 && sv_stride < (int64_t(1) << n)) return set_error(QGB_EINVAL, "state stride too small");
    if (mat_stride < 0) return set_error(QGB_EINVAL, "negative matrix stride");
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
    uint64_t in_tile = (L >= 64) ? ~0ull : ((1ull << L) - 1);
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
        if (k > kmax) kmax = k;
    }
    a.mat_stride = mat_stride;
    a.batch = batch;
    a.sv_stride = sv_stride;
    a.tiles = uint64_t(1) << (n - m);
    cudaStream_t st = (cudaStream_t)stream;
    return dtype == QGB_C64 ? dispatch_sweep<float>(sv, mats, a, kmax, st) : dispatch_sweep<double>(sv, mats, a, kmax, st);
}
