// Dense k-qubit gate application on the 5th-generation tensor cores
// (tcgen05, sm_103a), complex64, k = 4, 5, 6: one read and one write of the
// state per fused block, like dense_reg_kernel, but with the arithmetic moved
// off the FP32 pipes so that 6-qubit blocks (half the HBM passes of 4-qubit
// blocks) still run at memory speed.
//
// Replaces the reference's per-gate `op_action` (tensorQ/statevector_sim.py:124-140)
// for fused blocks of up to six qubits.
//
// Formulation. A group is the 2^k amplitudes that differ only in the target
// bits. For 128 groups at a time the kernel forms the real product
//     Y[128 x 2D] = X[128 x 2D] * W[2D x 2D],     D = 2^k,
// where row g of X holds group g's amplitudes as (re, im) pairs in memory
// order of the target bits, and W is the real form [[Mr, Mi], [-Mi, Mr]] of the
// (row/column permuted) gate matrix. That is 8 * D real flops per amplitude,
// the same count as the complex product.
//
// Precision. kind::tf32 multiplies 19-bit operands, so every operand is split
// as x = hi + lo with hi = x rounded to the nearest tf32 value and lo = x - hi
// (exact in fp32, |lo| <= 2^-11 |x|); Y = Xhi*Wlo + Xlo*Whi + Xhi*Whi with
// fp32 accumulation. The dropped Xlo*Wlo term and the tf32 reading of the lo
// parts are below 2^-21 relative each: the result agrees with an fp32 dot
// product to its own rounding level (about 1e-7 relative to the group norm).
//
// Data path per CTA (256 threads = 8 warps, one CTA per SM):
//   * tensor memory (TMEM) holds Xhi, Xlo (the A operands, lane = group row,
//     one 32-bit column per real component) and two accumulators D0/D1;
//   * shared memory holds Whi, Wlo as the B operand, K-major, no swizzle:
//     8-row x 16-byte core matrices, K-adjacent cores 128 B apart (leading
//     byte offset) and N-adjacent cores 256 B apart (stride byte offset);
//   * warps w and w+4 share TMEM lane quarter w (groups 32w..32w+31); warp
//     w+4h loads, splits and stores components [h*D/2, (h+1)*D/2) of its
//     group, and later reads the same half of the result row;
//   * a tile is 8192 amplitudes: 128 / (2D) blocks of 128 groups, each block
//     with its own Xhi, Xlo, D0, D1 columns (512 columns in all, any k);
//   * one thread issues the 3 * (2D/8) MMAs per block (M = 128, N = 2D, K = 8)
//     and commits them to an mbarrier; while they run, the CTA loads the tile
//     after next into registers (two register buffers) and drains the previous
//     tile's accumulator to HBM.
// Every wait on the mbarrier is bounded (about 2 s of %globaltimer); a wait
// that runs out sets a device status word read by qgb_check_status, and the
// CTA frees its tensor memory and returns.
#include <cstdio>
#include <cstdlib>

#include "qgb_common.cuh"

namespace qgb {

__device__ int g_tc_status = 0;

struct TcArgs {
    int k;
    int vec2;                         // 1: target bit 0 present, components (2m, 2m+1) adjacent
    int sorted[QGB_MAX_K];            // target bits, ascending
    int perm_in[1 << QGB_MAX_K];      // memory-order input component j -> matrix column
    int perm_out[1 << QGB_MAX_K];     // memory-order output component i -> matrix row
    uint64_t off[1 << (QGB_MAX_K - 1)];  // offsets of the low-half components (bits sorted[0..k-2])
    uint64_t hstride;                 // offset of the upper half (bit sorted[k-1])
    uint64_t tiles_per_state;         // groups / 128
    uint64_t tiles;                   // tiles_per_state * batch
    int64_t sv_stride;
};

constexpr int kTcThreads = 256;
constexpr unsigned long long kTcWaitNs = 2000000000ull;

template <int K> struct TcGeom {
    static constexpr int D = 1 << K;     // complex components per group
    static constexpr int H = D / 2;      // components per thread and group
    static constexpr int R = 2 * D;      // real width: MMA N and total K
    static constexpr int NB = 128 / R;   // 128-row blocks per tile: every tile is 8192 amplitudes (64 KB)
    static constexpr int BCOLS = 4 * R;  // TMEM columns per block: Xhi, Xlo, D0, D1
    static constexpr int NCOLS = NB * BCOLS;  // 512: one CTA per SM
    static constexpr uint32_t B_BYTES = uint32_t(R) * R * 4;
    static constexpr size_t SMEM = 2 * size_t(B_BYTES) + 128;
    // kind::tf32 instruction descriptor: f32 accumulator, tf32 A and B, both
    // K-major, N = R, M = 128.
    static constexpr uint32_t IDESC =
        (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(R >> 3) << 17) | (uint32_t(128 >> 4) << 24);
    static_assert(R >= 32 && R <= 256 && (R % 16) == 0, "MMA N out of range");
    static_assert(NCOLS == 512, "tensor memory holds 512 columns");
};

__device__ __forceinline__ uint32_t tc_smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ unsigned long long tc_global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool tc_wait_bounded(uint32_t bar, uint32_t parity) {
    const unsigned long long t0 = tc_global_ns();
    while (true) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar), "r"(parity), "r"(20000)
            : "memory");
        if (done) return true;
        if (tc_global_ns() - t0 > kTcWaitNs) return false;
    }
}

// Nearest tf32 value (ties away from zero), low 13 bits cleared.
__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r & 0xffffe000u);
}

// Byte offset of element (n, k) of a B operand with R rows (N) in the K-major
// no-swizzle layout: per K-step of 8 a block of R * 32 bytes; inside it core
// matrix (n / 8, (k % 8) / 4) at 256 * (n / 8) + 128 * ((k % 8) / 4).
__device__ __forceinline__ uint32_t b_off(int n, int k, int R) {
    return uint32_t((k >> 3) * (R * 32) + (n >> 3) * 256 + ((k >> 2) & 1) * 128 + (n & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint64_t b_desc(uint32_t addr) {
    return uint64_t((addr & 0x3FFFFu) >> 4) | (uint64_t(128 >> 4) << 16) | (uint64_t(256 >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{ .reg .pred p; setp.ne.b32 p, %4, 0; "
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p; }" ::"r"(d),
        "r"(a), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float* v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16};" ::"r"(taddr),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
        "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
        : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]), "=f"(v[8]),
          "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
        : "r"(taddr)
        : "memory");
    // The loaded registers are valid only after wait::ld; tying them to the
    // wait keeps every use behind it.
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7]),
                   "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]), "+f"(v[12]), "+f"(v[13]), "+f"(v[14]), "+f"(v[15])
                 :
                 : "memory");
}

template <int K>
__global__ void __launch_bounds__(kTcThreads, 1) dense_tc_kernel(float2* __restrict__ sv, const float2* __restrict__ op,
                                                                 const __grid_constant__ TcArgs a) {
    using G = TcGeom<K>;
    constexpr int D = G::D, H = G::H, R = G::R, NB = G::NB, BC = G::BCOLS;
    extern __shared__ unsigned char tc_smem_raw[];
    unsigned char* sb = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 127) & ~uintptr_t(127));
    unsigned char* Bhi = sb;
    unsigned char* Blo = sb + G::B_BYTES;
    __shared__ __align__(8) uint64_t mma_bar;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q = warp & 3, h = warp >> 2;

    // B operand: W = [[Mr, Mi], [-Mi, Mr]] in (output, input) memory order, split hi/lo.
    for (int p = tid; p < D * D; p += kTcThreads) {
        const int i = p / D, j = p - (p / D) * D;
        const float2 m = op[a.perm_out[i] * D + a.perm_in[j]];
        const float w[4] = {m.x, -m.y, m.y, m.x};  // (2i,2j) (2i,2j+1) (2i+1,2j) (2i+1,2j+1)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const uint32_t o = b_off(2 * i + (e >> 1), 2 * j + (e & 1), R);
            const float hi = tf32_hi(w[e]);
            *reinterpret_cast<float*>(Bhi + o) = hi;
            *reinterpret_cast<float*>(Blo + o) = w[e] - hi;
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_u32(&tmem_slot)),
                     "r"(G::NCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 32) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem_u32(&mma_bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t bar = tc_smem_u32(&mma_bar);
    const uint32_t row = tmem + (uint32_t(32 * q) << 16);  // this warp's lane quarter
    const uint32_t bhi = tc_smem_u32(Bhi), blo = tc_smem_u32(Blo);
    // TMEM columns of block bk: Xhi at bk*BC, Xlo at bk*BC + R, accumulators at bk*BC + 2R + buf*R.

    auto group_ptr = [&](uint64_t t, int bk) -> float2* {
        const uint64_t b = t / a.tiles_per_state, tt = t - b * a.tiles_per_state;
        const uint64_t g = (tt * NB + uint64_t(bk)) * 128 + uint64_t(32 * q + lane);
        return sv + int64_t(b) * a.sv_stride + insert_zeros(g, a.sorted, K) + uint64_t(h) * a.hstride;
    };
    using Buf = float2[NB][H];
    auto load = [&](uint64_t t, Buf& v) {
#pragma unroll
        for (int bk = 0; bk < NB; ++bk) {
            const float2* p = group_ptr(t, bk);
            if (a.vec2) {
#pragma unroll
                for (int m = 0; m < H / 2; ++m) {
                    const float4 x = *reinterpret_cast<const float4*>(p + a.off[2 * m]);
                    v[bk][2 * m] = make_float2(x.x, x.y);
                    v[bk][2 * m + 1] = make_float2(x.z, x.w);
                }
            } else {
#pragma unroll
                for (int j = 0; j < H; ++j) v[bk][j] = p[a.off[j]];
            }
        }
    };
    auto store_x = [&](const Buf& v) {
#pragma unroll
        for (int bk = 0; bk < NB; ++bk) {
#pragma unroll
            for (int c0 = 0; c0 < D; c0 += 16) {
                float hi[16], lo[16];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const float2 x = v[bk][c0 / 2 + e];
                    hi[2 * e] = tf32_hi(x.x);
                    hi[2 * e + 1] = tf32_hi(x.y);
                    lo[2 * e] = x.x - hi[2 * e];
                    lo[2 * e + 1] = x.y - hi[2 * e + 1];
                }
                tmem_st16(row + uint32_t(bk * BC + h * D + c0), hi);
                tmem_st16(row + uint32_t(bk * BC + R + h * D + c0), lo);
            }
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    };
    auto issue = [&](int buf) {
        tc_fence_after();
#pragma unroll 1
        for (int bk = 0; bk < NB; ++bk) {
            const uint32_t d = tmem + uint32_t(bk * BC + 2 * R + buf * R);
            const uint32_t xh = tmem + uint32_t(bk * BC), xl = xh + R;
#pragma unroll 1
            for (int s = 0; s < R / 8; ++s)
                tc_mma(d, xh + uint32_t(8 * s), b_desc(blo + uint32_t(s * R * 32)), G::IDESC, s > 0);
#pragma unroll 1
            for (int s = 0; s < R / 8; ++s)
                tc_mma(d, xl + uint32_t(8 * s), b_desc(bhi + uint32_t(s * R * 32)), G::IDESC, 1);
#pragma unroll 1
            for (int s = 0; s < R / 8; ++s)
                tc_mma(d, xh + uint32_t(8 * s), b_desc(bhi + uint32_t(s * R * 32)), G::IDESC, 1);
        }
        tc_commit(bar);
    };
    auto drain = [&](uint64_t t, int buf) {
#pragma unroll
        for (int bk = 0; bk < NB; ++bk) {
            float2* p = group_ptr(t, bk);
#pragma unroll
            for (int c0 = 0; c0 < D; c0 += 16) {
                float r[16];
                tmem_ld16(row + uint32_t(bk * BC + 2 * R + buf * R + h * D + c0), r);
                if (a.vec2) {
#pragma unroll
                    for (int m = 0; m < 4; ++m)
                        *reinterpret_cast<float4*>(p + a.off[c0 / 2 + 2 * m]) =
                            make_float4(r[4 * m], r[4 * m + 1], r[4 * m + 2], r[4 * m + 3]);
                } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e) p[a.off[c0 / 2 + e]] = make_float2(r[2 * e], r[2 * e + 1]);
                }
            }
        }
    };

    // Software pipeline over this CTA's tiles t0, t0 + step, ...: while the
    // tensor cores work on tile t, the registers receive tile t + 2 step and
    // the accumulator of tile t - step drains to HBM; tile t + step (loaded one
    // stage earlier) is staged into TMEM as soon as tile t's MMAs complete.
    const uint64_t step = gridDim.x;
    uint64_t t = blockIdx.x;  // the grid never exceeds the tile count
    Buf vA, vB;
    load(t, vA);
    store_x(vA);
    tc_fence_before();
    __syncthreads();
    if (tid == 0) issue(0);
    if (t + step < a.tiles) load(t + step, vB);
    uint64_t prev = 0;
    bool have_prev = false;
    int buf = 0;
    uint32_t phase = 0;
    // On entry: tile t's MMAs run into accumulator `buf`; `nxt` holds (or is
    // receiving) tile t + step; `cur` is free. Returns false after the last tile.
    auto stage = [&](Buf& cur, Buf& nxt) -> bool {
        const uint64_t tn = t + step, tnn = tn + step;
        if (tnn < a.tiles) load(tnn, cur);
        if (have_prev) drain(prev, buf ^ 1);
        const bool ok = tc_wait_bounded(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(&g_tc_status, 1);
            return false;
        }
        tc_fence_after();
        if (tn >= a.tiles) {
            drain(t, buf);
            return false;
        }
        store_x(nxt);  // tile t's MMAs are done: X may be overwritten
        tc_fence_before();
        __syncthreads();
        if (tid == 0) issue(buf ^ 1);
        prev = t;
        have_prev = true;
        t = tn;
        buf ^= 1;
        return true;
    };
    while (stage(vA, vB) && stage(vB, vA)) {
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(G::NCOLS) : "memory");
    }
}

}  // namespace qgb

using namespace qgb;

namespace {

int g_dense_impl = -1;  // -1: not read yet; 0: CUDA cores only; 1: tensor cores for k = 5, 6; 2: also k = 4

int dense_impl() {
    if (g_dense_impl < 0) {
        const char* e = getenv("QGB_DENSE_IMPL");
        g_dense_impl = 2;
        if (e && (e[0] == '0' || e[0] == 'c')) g_dense_impl = 0;
        if (e && e[0] == '1') g_dense_impl = 1;
    }
    return g_dense_impl;
}

template <int K>
int launch_tc(float2* sv, const float2* op, const TcArgs& a, cudaStream_t st) {
    using G = TcGeom<K>;
    static int per_sm = 0;
    if (per_sm == 0) {
        if (cudaFuncSetAttribute(dense_tc_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(G::SMEM)) !=
            cudaSuccess)
            return qgb_host::check_launch("dense_tc attribute");
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dense_tc_kernel<K>, kTcThreads, G::SMEM) != cudaSuccess)
            return qgb_host::check_launch("dense_tc occupancy");
        per_sm = occ < 1 ? occ : 1;  // each CTA holds all 512 TMEM columns
        if (per_sm < 1) return qgb_host::set_error(QGB_ECUDA, "dense_tc kernel does not fit on an SM");
    }
    const uint64_t cap = uint64_t(qgb_host::sm_count()) * uint64_t(per_sm);
    const unsigned grid = unsigned(a.tiles < cap ? a.tiles : cap);
    dense_tc_kernel<K><<<grid, kTcThreads, G::SMEM, st>>>(sv, op, a);
    return qgb_host::check_launch("dense_tc kernel");
}

}  // namespace

namespace qgb_host {

int tc_status_read_clear() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, qgb::g_tc_status, sizeof(int)) != cudaSuccess) return -1;
    if (v != 0) {
        const int z = 0;
        cudaMemcpyToSymbol(qgb::g_tc_status, &z, sizeof(int));
    }
    return v;
}

int set_dense_impl(int mode) {
    if (mode < 0 || mode > 2) return set_error(QGB_EINVAL, "dense implementation %d unknown (0, 1, 2)", mode);
    g_dense_impl = mode;
    return QGB_OK;
}

// Tensor-core path for a complex64 dense op; returns QGB_EDECLINE (and touches
// nothing) when the op is not one it takes, so that the caller runs the
// CUDA-core kernel instead.
int try_dense_tc(void* sv, const void* op, int nbits, const int* sorted, const int* in_bits, const int* out_bits,
                 int k, int64_t op_stride, int64_t batch, int64_t sv_stride, cudaStream_t st) {
    const int mode = dense_impl();
    if (mode == 0 || k < 4 || k > 6 || (k == 4 && mode < 2)) return QGB_EDECLINE;
    if (nbits < 13) return QGB_EDECLINE;              // fewer than one 8192-amplitude tile
    if (batch > 1 && op_stride != 0) return QGB_EDECLINE;  // one operator for the whole batch
    TcArgs a{};
    a.k = k;
    for (int j = 0; j < k; ++j) a.sorted[j] = sorted[j];
    const int D = 1 << k;
    uint64_t scat[1 << QGB_MAX_K];
    for (int j = 0; j < D; ++j) {
        uint64_t o = 0;
        for (int i = 0; i < k; ++i)
            if ((j >> i) & 1) o |= uint64_t(1) << sorted[i];
        scat[j] = o;
    }
    for (int j = 0; j < D / 2; ++j) a.off[j] = scat[j];
    a.hstride = uint64_t(1) << sorted[k - 1];
    for (int c = 0; c < D; ++c) {
        const uint64_t oi = matrix_offset(c, in_bits, k), oo = matrix_offset(c, out_bits, k);
        for (int j = 0; j < D; ++j) {
            if (scat[j] == oi) a.perm_in[j] = c;
            if (scat[j] == oo) a.perm_out[j] = c;
        }
    }
    a.vec2 = sorted[0] == 0 ? 1 : 0;
    if (a.vec2 && ((reinterpret_cast<uintptr_t>(sv) % 16) || (batch > 1 && (sv_stride % 2)))) a.vec2 = 0;
    a.tiles_per_state = uint64_t(1) << (nbits - 13);  // 8192 amplitudes per tile
    a.tiles = a.tiles_per_state * uint64_t(batch);
    a.sv_stride = batch > 1 ? sv_stride : 0;
    float2* s = static_cast<float2*>(sv);
    const float2* m = static_cast<const float2*>(op);
    switch (k) {
        case 4: return launch_tc<4>(s, m, a, st);
        case 5: return launch_tc<5>(s, m, a, st);
        default: return launch_tc<6>(s, m, a, st);
    }
}

}  // namespace qgb_host

extern "C" int qgb_set_dense_impl(int mode) { return qgb_host::set_dense_impl(mode); }

extern "C" int qgb_get_dense_impl(void) { return dense_impl(); }
