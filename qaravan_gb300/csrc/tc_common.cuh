// Pieces shared by the tensor-core kernels (dense_tc.cu, tc_sweep.cu):
// shared-memory and tensor-memory addressing, the tile swizzle, cp.async,
// named barriers of the data warps, packed f32x2 arithmetic, the fp16 hi/lo
// split, tcgen05 MMA / commit / load / store wrappers and the bounded
// mbarrier wait.
#pragma once

#include <cuda_fp16.h>

#include "qgb_common.cuh"

namespace qgb {

constexpr unsigned long long kTcWaitNs = 2000000000ull;  // bounded mbarrier waits: about 2 s

constexpr int kChainEpoch = 4;                 // passes per norm-chain epoch
constexpr int kTcDataThreads = 256;           // 8 data warps
constexpr int kTcThreads = kTcDataThreads + 32;  // + the MMA warp

struct TcArgs {
    int k;
    int vec2;                            // global bit 0 is a target: components (2m, 2m+1) adjacent
    int vec4;                            // global bits 0 and 1 are targets: rows are runs of >= 4 components
    int L;                               // tile bits 0..L-1 are global bits 0..L-1 (L >= 7)
    int tile_bits[13];                   // global bit of each tile bit, ascending
    int pos_g[13];                       // tile positions of the 13 - k group bits, ascending
    int perm_in[1 << QGB_MAX_K];         // memory-order input component j -> matrix column
    int perm_out[1 << QGB_MAX_K];        // memory-order output component i -> matrix row
    uint32_t uts[1 << (QGB_MAX_K - 1)];  // swizzled tile-index offsets of the low-half components
    uint32_t ut_h;                       // tile-index offset of the upper half (target sorted[k-1])
    uint64_t g512[16];                   // global offset of tile index 512 m
    uint64_t off[1 << (QGB_MAX_K - 1)];  // global offsets of the low-half components
    uint64_t hstride;                    // global offset of the upper half
    uint64_t hoff[64];                   // global offset of tile bits L..12, indexed by u >> L
    uint64_t tiles_per_state;            // 2^(n - 13)
    uint64_t tiles;                      // tiles_per_state * batch
    int64_t sv_stride;
    double* chain;                       // norm chain (3 slots of {reference, output} squared norms) or null
    const double* scale;                 // MODE 0: device factor f, the op applied is f * M (null: 1)
    int c_prev, c_cur, c_next;           // slots of the previous epoch, this epoch, the next epoch (-1: none)
    int c_head, c_tail;                  // this pass opens its epoch (corrects) / closes it (measures its output)
};

template <int K> struct TcGeom {
    static constexpr int D = 1 << K;     // complex components per group
    static constexpr int H = D / 2;      // components per thread and group
    static constexpr int R = 2 * D;      // real width: MMA N and total K
    static constexpr int NB = 128 / R;   // 128-row blocks per tile: every tile is 8192 amplitudes (64 KB)
    static constexpr int BCOLS = 4 * R;  // TMEM columns per block: X0 (hi, lo), X1 (hi, lo), D0, D1
    static constexpr int NCOLS = NB * BCOLS;  // 512: one CTA per SM
    static constexpr uint32_t B_BYTES = uint32_t(R) * R * 2;
    static constexpr uint32_t TILE_BYTES = 8192 * 8;
    static constexpr uint32_t STAGE_BYTES = 8 * 2048;  // per data warp: 32 rows x 8 components of output
    static constexpr size_t SMEM = 2 * size_t(B_BYTES) + 2 * size_t(TILE_BYTES) + STAGE_BYTES + 128;
    // kind::f16 instruction descriptor: f32 accumulator, f16 A and B, both
    // K-major, N = R, M = 128.
    static constexpr uint32_t IDESC = (1u << 4) | (uint32_t(R >> 3) << 17) | (uint32_t(128 >> 4) << 24);
    static_assert(R >= 32 && R <= 256 && (R % 16) == 0, "MMA N out of range");
    static_assert(NCOLS == 512, "tensor memory holds 512 columns");
};

__device__ __forceinline__ uint32_t tc_smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ bool tc_wait_bounded(uint32_t bar, uint32_t parity) {
    return mbar_wait_parity_bounded(bar, parity, kTcWaitNs);
}

// The same bounded wait by polling (mbarrier.test_wait, no suspension): for
// waits on the critical path of a pipeline, where a suspended thread's wake-up
// would add to every step. The time limit is checked every 256 polls.
__device__ __forceinline__ bool tc_spin_bounded(uint32_t bar, uint32_t parity) {
    const unsigned long long t0 = global_ns();
    for (uint32_t i = 0;; ++i) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((i & 255u) == 255u && global_ns() - t0 > kTcWaitNs) return false;
    }
}

// Byte offset of fp16 element (n, k) of a B operand with R rows (N) in the
// K-major no-swizzle layout: per K-step of 16 a block of R * 32 bytes; inside
// it core matrix (n / 8, (k % 16) / 8) at 256 * (n / 8) + 128 * ((k % 16) / 8).
__device__ __forceinline__ uint32_t b_off(int n, int k, int R) {
    return uint32_t((k >> 4) * (R * 32) + (n >> 3) * 256 + ((k >> 3) & 1) * 128 + (n & 7) * 16 + (k & 7) * 2);
}

// Word (8-byte amplitude) index of tile index u in a staged tile: the 16-byte
// granule index (bits 1..3) is XORed with a fold of the higher bits, so the 32
// lanes reading one component of 32 rows hit distinct banks whether the rows
// differ in low or in high tile bits. Bit 0 is left alone: a 16-byte granule
// (two amplitudes) stays whole, as cp.async copies it. The map is linear over
// XOR, so swz(a | b) = swz(a) ^ swz(b) for disjoint bit sets: row and
// component parts are swizzled once and combined with one XOR.
__host__ __device__ __forceinline__ uint32_t tile_swz(uint32_t u) {
    return u ^ ((((u >> 4) ^ (u >> 7) ^ (u >> 10)) & 7u) << 1);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

__device__ __forceinline__ void data_bar() { asm volatile("bar.sync 5, 256;" ::: "memory"); }
__device__ __forceinline__ bool data_bar_any(bool v) {
    uint32_t r;
    asm volatile("{ .reg .pred p, q; setp.ne.u32 p, %1, 0; bar.red.or.pred q, 5, 256, p; selp.u32 %0, 1, 0, q; }"
                 : "=r"(r)
                 : "r"(uint32_t(v))
                 : "memory");
    return r != 0;
}

// Packed pairs of fp32 (one 64-bit register, Blackwell's f32x2 arithmetic).
__device__ __forceinline__ unsigned long long f2pack(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2unpack(unsigned long long v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2fma(unsigned long long a, unsigned long long b, unsigned long long c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ unsigned long long f2mul(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

// Sum of squares of N floats (N a multiple of 8) with 8 interleaved partial
// sums (shallower rounding-error growth than one running sum), two per f32x2.
template <int N> __device__ __forceinline__ float sumsq8(const float* x) {
    unsigned long long acc[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll
    for (int i = 0; i < N / 2; ++i) {
        const unsigned long long v = f2pack(x[2 * i], x[2 * i + 1]);
        acc[i & 3] = f2fma(v, v, acc[i & 3]);
    }
    float s[8];
#pragma unroll
    for (int j = 0; j < 4; ++j) f2unpack(acc[j], s[2 * j], s[2 * j + 1]);
    return ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// 2^e for e in [-126, 127].
__device__ __forceinline__ float exp2i(int e) { return __uint_as_float(uint32_t(e + 127) << 23); }

// Scale exponent s with max 2^s in [2^14, 2^15) for a non-negative maximum m
// (clamped to [-100, 100]; zero rows get 100 and stay zero).
__device__ __forceinline__ int scale_exp(float m) {
    const int s = 141 - int((__float_as_uint(m) >> 23) & 0xffu);
    return s < -100 ? -100 : (s > 100 ? 100 : s);
}

// (a, b) -> packed fp16 pair hi and the packed rounding remainders lo.
__device__ __forceinline__ void split_f16(float a, float b, uint32_t& hi, uint32_t& lo) {
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// The B operand W = [[Mr, Mi], [-Mi, Mr]] of a 2^K x 2^K complex op (rows in
// output memory order perm_out, columns in input order perm_in), scaled by the
// power of two 2^sw that brings its largest entry into [2^14, 2^15), times
// 1 + gcorr when gcorr != 0, split into fp16 hi and lo planes in the K-major
// core-matrix layout of b_off. All nthr threads of the CTA take part (two
// CTA barriers inside; *wmax_bits must be zero and visible to all threads on
// entry). Each thread loads all its entries before using any -- one round of
// L2 latency instead of one per entry -- and writes whole 16-byte core-matrix
// rows (8 fp16 of one row); the values are those of an entry-by-entry build.
// Returns sw.
template <int K, int NTHR>
__device__ __forceinline__ int tc_build_w(unsigned char* Bhi, unsigned char* Blo, const float2* __restrict__ op,
                                          const int* perm_out, const int* perm_in, float gcorr,
                                          uint32_t* wmax_bits, int tid) {
    constexpr int D = 1 << K, R = 2 * D;
    constexpr int NI = D * (D / 4);               // (complex row i, group c of 4 complex columns)
    constexpr int IT = (NI + NTHR - 1) / NTHR;
    float2 v[IT][4];
    float m = 0.f;
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int q = tid + it * NTHR;
        if (q < NI) {
            const int i = q & (D - 1), c = q >> K;
            const float2* row = op + perm_out[i] * D;
#pragma unroll
            for (int t = 0; t < 4; ++t) v[it][t] = row[perm_in[4 * c + t]];
#pragma unroll
            for (int t = 0; t < 4; ++t) m = fmaxf(m, fmaxf(fabsf(v[it][t].x), fabsf(v[it][t].y)));
        }
    }
    atomicMax(wmax_bits, __float_as_uint(m));
    __syncthreads();
    const int sw = scale_exp(__uint_as_float(*wmax_bits));
    const float wscale = exp2i(sw);
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int q = tid + it * NTHR;
        if (q < NI) {
            const int i = q & (D - 1), c = q >> K;
            uint32_t h0[4], l0[4], h1[4], l1[4];  // real rows 2i (Mr, -Mi) and 2i + 1 (Mi, Mr)
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                float w[4] = {v[it][t].x * wscale, -v[it][t].y * wscale, v[it][t].y * wscale, v[it][t].x * wscale};
                if (gcorr != 0.f) {
#pragma unroll
                    for (int e = 0; e < 4; ++e) w[e] = fmaf(w[e], gcorr, w[e]);
                }
                split_f16(w[0], w[1], h0[t], l0[t]);
                split_f16(w[2], w[3], h1[t], l1[t]);
            }
            // b_off(n, 8 c, R): the core-matrix row of real row n and columns 8c .. 8c + 7
            const uint32_t o0 = uint32_t((c >> 1) * (R * 32) + ((2 * i) >> 3) * 256 + (c & 1) * 128 + ((2 * i) & 7) * 16);
            const uint32_t o1 = o0 + 16;  // row 2i + 1: the next row of the same core matrix
            *reinterpret_cast<uint4*>(Bhi + o0) = make_uint4(h0[0], h0[1], h0[2], h0[3]);
            *reinterpret_cast<uint4*>(Blo + o0) = make_uint4(l0[0], l0[1], l0[2], l0[3]);
            *reinterpret_cast<uint4*>(Bhi + o1) = make_uint4(h1[0], h1[1], h1[2], h1[3]);
            *reinterpret_cast<uint4*>(Blo + o1) = make_uint4(l1[0], l1[1], l1[2], l1[3]);
        }
    }
    return sw;
}

__device__ __forceinline__ uint64_t b_desc(uint32_t addr) {
    return uint64_t((addr & 0x3FFFFu) >> 4) | (uint64_t(128 >> 4) << 16) | (uint64_t(256 >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{ .reg .pred p; setp.ne.b32 p, %4, 0; "
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p; }" ::"r"(d),
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

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t* v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr), "r"(v[0]),
                 "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
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

// 32 and 64 columns in one load and one wait (a half row of a 5- or 6-qubit
// block's accumulator), so a drain makes one tensor-memory round trip.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]), "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15]), "=f"(v[16]), "=f"(v[17]), "=f"(v[18]), "=f"(v[19]), "=f"(v[20]), "=f"(v[21]), "=f"(v[22]), "=f"(v[23]), "=f"(v[24]), "=f"(v[25]), "=f"(v[26]), "=f"(v[27]), "=f"(v[28]), "=f"(v[29]), "=f"(v[30]), "=f"(v[31])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7]), "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]), "+f"(v[12]), "+f"(v[13]), "+f"(v[14]), "+f"(v[15]), "+f"(v[16]), "+f"(v[17]), "+f"(v[18]), "+f"(v[19]), "+f"(v[20]), "+f"(v[21]), "+f"(v[22]), "+f"(v[23]), "+f"(v[24]), "+f"(v[25]), "+f"(v[26]), "+f"(v[27]), "+f"(v[28]), "+f"(v[29]), "+f"(v[30]), "+f"(v[31])
                 :
                 : "memory");
}
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float* v) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]), "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15]), "=f"(v[16]), "=f"(v[17]), "=f"(v[18]), "=f"(v[19]), "=f"(v[20]), "=f"(v[21]), "=f"(v[22]), "=f"(v[23]), "=f"(v[24]), "=f"(v[25]), "=f"(v[26]), "=f"(v[27]), "=f"(v[28]), "=f"(v[29]), "=f"(v[30]), "=f"(v[31]), "=f"(v[32]), "=f"(v[33]), "=f"(v[34]), "=f"(v[35]), "=f"(v[36]), "=f"(v[37]), "=f"(v[38]), "=f"(v[39]), "=f"(v[40]), "=f"(v[41]), "=f"(v[42]), "=f"(v[43]), "=f"(v[44]), "=f"(v[45]), "=f"(v[46]), "=f"(v[47]), "=f"(v[48]), "=f"(v[49]), "=f"(v[50]), "=f"(v[51]), "=f"(v[52]), "=f"(v[53]), "=f"(v[54]), "=f"(v[55]), "=f"(v[56]), "=f"(v[57]), "=f"(v[58]), "=f"(v[59]), "=f"(v[60]), "=f"(v[61]), "=f"(v[62]), "=f"(v[63])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7]), "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]), "+f"(v[12]), "+f"(v[13]), "+f"(v[14]), "+f"(v[15]), "+f"(v[16]), "+f"(v[17]), "+f"(v[18]), "+f"(v[19]), "+f"(v[20]), "+f"(v[21]), "+f"(v[22]), "+f"(v[23]), "+f"(v[24]), "+f"(v[25]), "+f"(v[26]), "+f"(v[27]), "+f"(v[28]), "+f"(v[29]), "+f"(v[30]), "+f"(v[31]), "+f"(v[32]), "+f"(v[33]), "+f"(v[34]), "+f"(v[35]), "+f"(v[36]), "+f"(v[37]), "+f"(v[38]), "+f"(v[39]), "+f"(v[40]), "+f"(v[41]), "+f"(v[42]), "+f"(v[43]), "+f"(v[44]), "+f"(v[45]), "+f"(v[46]), "+f"(v[47]), "+f"(v[48]), "+f"(v[49]), "+f"(v[50]), "+f"(v[51]), "+f"(v[52]), "+f"(v[53]), "+f"(v[54]), "+f"(v[55]), "+f"(v[56]), "+f"(v[57]), "+f"(v[58]), "+f"(v[59]), "+f"(v[60]), "+f"(v[61]), "+f"(v[62]), "+f"(v[63])
                 :
                 : "memory");
}

template <int N> __device__ __forceinline__ void tmem_ld_row(uint32_t taddr, float* v) {
    static_assert(N == 16 || N == 32 || N == 64, "row width");
    if constexpr (N == 16) tmem_ld16(taddr, v);
    else if constexpr (N == 32) tmem_ld32(taddr, v);
    else tmem_ld64(taddr, v);
}

}  // namespace qgb

namespace qgb_host {
// dense_tc.cu: the geometry of one tensor-core pass (also used by the batched kernels)
int build_tc_args(qgb::TcArgs& a, int nbits, const int* sorted, const int* in_bits, const int* out_bits, int k,
                  int64_t batch, int64_t sv_stride);
}  // namespace qgb_host
