// Shared device/host helpers of the gate-application engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qgb.h"

namespace qgb {

template <typename T> struct CplxOf;
template <> struct CplxOf<float> { using type = float2; };
template <> struct CplxOf<double> { using type = double2; };
template <typename T> using cplx = typename CplxOf<T>::type;

template <typename T> __host__ __device__ __forceinline__ cplx<T> mk(T re, T im) {
    cplx<T> r;
    r.x = re;
    r.y = im;
    return r;
}

// acc += a * b (complex), four fused multiply-adds.
template <typename C> __device__ __forceinline__ void cfma(C& acc, const C& a, const C& b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}

// ---- bounded device waits --------------------------------------------------
// Every wait in the library's kernels gives up after a time limit (read from
// %globaltimer) instead of spinning forever: the caller then records a status
// word that the host reads (qgb_check_status -> QGB_ETIMEOUT) and returns.

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for phase `parity` of the shared-memory mbarrier at `bar`; false after limit_ns.
__device__ __forceinline__ bool mbar_wait_parity_bounded(uint32_t bar, uint32_t parity,
                                                         unsigned long long limit_ns) {
    const unsigned long long t0 = global_ns();
    while (true) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar), "r"(parity), "r"(20000)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// Waits until the global int at `flag` equals `want`; false after limit_ns.
__device__ __forceinline__ bool flag_wait_bounded(const volatile int* flag, int want, unsigned long long limit_ns) {
    const unsigned long long t0 = global_ns();
    while (*flag != want) {
        __nanosleep(1000);
        if (global_ns() - t0 > limit_ns) return false;
    }
    return true;
}

// Insert a zero at each (ascending) bit position of `sorted_bits`.
__device__ __forceinline__ uint64_t insert_zeros(uint64_t g, const int* sorted_bits, int k) {
#pragma unroll 6
    for (int j = 0; j < k; ++j) {
        const int b = sorted_bits[j];
        const uint64_t lo = g & ((uint64_t(1) << b) - 1);
        g = ((g >> b) << (b + 1)) | lo;
    }
    return g;
}

// Scatter the low bits of `v` to the listed bit positions (ascending list).
__device__ __forceinline__ uint64_t scatter_bits(uint64_t v, const int* bits, int nb) {
    uint64_t out = 0;
    for (int j = 0; j < nb; ++j) out |= ((v >> j) & 1ull) << bits[j];
    return out;
}

// Offset of matrix row/column r in the state: bit (k-1-j) of r goes to bit pos[j].
// Accumulators of many float partial sums kept on the FP32 pipe: a float sum with
// its compensation term (Kahan summation: the error stays at a few float
// roundings of the summed magnitudes, however many terms), and float64 for
// double data. GB300's FP64 pipe is narrow: a float64 add per warp and op in an
// inner loop stalls the warps that issue it.
struct WAccF {
    float s, c;
};
template <typename T> struct WAccOf { using type = double; };
template <> struct WAccOf<float> { using type = WAccF; };
static_assert(sizeof(WAccF) == sizeof(double), "accumulator layout");

__device__ __forceinline__ void wacc_add(double& a, double v) { a += v; }
__device__ __forceinline__ void wacc_add(WAccF& a, float v) {
    const float y = __fsub_rn(v, a.c);
    const float t = __fadd_rn(a.s, y);
    a.c = __fsub_rn(__fsub_rn(t, a.s), y);
    a.s = t;
}
__device__ __forceinline__ double wacc_value(const double& a) { return a; }
__device__ __forceinline__ double wacc_value(const WAccF& a) { return double(a.s) - double(a.c); }
__device__ __forceinline__ void wacc_zero(double& a) { a = 0.0; }
__device__ __forceinline__ void wacc_zero(WAccF& a) {
    a.s = 0.f;
    a.c = 0.f;
}

__host__ __device__ __forceinline__ uint64_t matrix_offset(int r, const int* pos, int k) {
    uint64_t off = 0;
    for (int j = 0; j < k; ++j) off |= uint64_t((r >> (k - 1 - j)) & 1) << pos[j];
    return off;
}

// Shared-memory swizzle for a staged tile, on 16-byte granules: the 16-byte
// chunk index has bits 3..5 XORed into bits 0..2, which spreads the amplitudes
// a warp touches over the 32 banks when the gate acts on the tile's low bits.
template <typename T> __device__ __forceinline__ uint32_t swz(uint32_t e);
template <> __device__ __forceinline__ uint32_t swz<float>(uint32_t e) { return e ^ (((e >> 4) & 7u) << 1); }
template <> __device__ __forceinline__ uint32_t swz<double>(uint32_t e) { return e ^ ((e >> 3) & 7u); }

// Per-thread accumulators. complex128 states sum in float64 throughout. For
// complex64 states the products and the running sums are float32 in two
// levels -- chunks of kChunk grid-stride iterations, kChunk chunks summed into
// a second float32 sum -- which is then folded into a float64 sum: the FP64
// pipe of this part runs at a small fraction of its FP32 rate, and float64
// arithmetic on every element (conversions included), or even once per chunk,
// kept these kernels bound by that pipe far below HBM speed. Each level of
// kChunk float32 terms carries a relative error of at most kChunk * 2^-24 of
// the sum of the magnitudes (well inside complex64 tolerances); the order stays
// fixed, so results remain bitwise reproducible.
constexpr int kChunk = 16;

template <typename T, int NV>
struct Acc {
    double d[NV];
    __device__ __forceinline__ Acc() {
#pragma unroll
        for (int j = 0; j < NV; ++j) d[j] = 0.0;
    }
    __device__ __forceinline__ void add(int j, double v) { d[j] += v; }
    __device__ __forceinline__ void step() {}
    __device__ __forceinline__ void flush() {}
};

template <int NV>
struct Acc<float, NV> {
    double d[NV];
    float f[NV], g[NV];
    int cnt, cnt2;
    __device__ __forceinline__ Acc() : cnt(0), cnt2(0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            d[j] = 0.0;
            f[j] = g[j] = 0.0f;
        }
    }
    __device__ __forceinline__ void add(int j, float v) { f[j] += v; }
    // the chunk into the second level
    __device__ __forceinline__ void chunk() {
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            g[j] += f[j];
            f[j] = 0.0f;
        }
        cnt = 0;
    }
    __device__ __forceinline__ void flush() {
        chunk();
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            d[j] += double(g[j]);
            g[j] = 0.0f;
        }
        cnt2 = 0;
    }
    __device__ __forceinline__ void step() {
        if (++cnt == kChunk) {
            if (++cnt2 == kChunk) flush();
            else chunk();
        }
    }
};

}  // namespace qgb

// ---- host-side helpers shared by the translation units -------------------
namespace qgb_host {
int set_error(int code, const char* fmt, ...);
int check_launch(const char* what);
int sm_count();
// Internal status (never returned through the C ABI): a specialised kernel
// declines an op, and the caller runs the general kernel instead.
constexpr int QGB_EDECLINE = 1000;
int try_dense_tc(void* sv, const void* op, int nbits, const int* sorted, const int* in_bits, const int* out_bits,
                 int k, int64_t op_stride, int64_t batch, int64_t sv_stride, int unitary, cudaStream_t st,
                 double* chain = nullptr, int link = 0, const double* scale = nullptr);
int tc_status_read_clear();
int tcs_status_read_clear();
int dmb_status_read_clear();
int traj_status_read_clear();
int fuse_status_read_clear();
}  // namespace qgb_host
