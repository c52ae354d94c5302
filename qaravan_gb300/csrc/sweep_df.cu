// complex128 tile sweeps in double-float arithmetic.
//
// GB300's FP64 pipe runs at about 1/62 of its FP32 rate (1.26 vs 78.5 TFLOP/s
// measured with qgb_fma_probe), and the float64 sweep kernel sits at that
// FP64 limit, far below HBM speed. Here a complex128 tile is converted, once it
// is in shared memory, to double-float numbers (each float64 component x as a
// pair of floats h + l carrying 48 significant bits), every op of the sweep is
// applied with FP32 instructions only, and the tile is converted back to
// float64 on its way out. The state in HBM stays complex128 (double2) between
// passes, so every other kernel reads it unchanged.
//
// Arithmetic (Dekker's product and Knuth's two-sum, the double-float scheme of
// Hida, Li & Bailey's QD library, restated): a product a*b of two pairs is the
// float product p = ah*bh, its exact rounding error fma(ah, bh, -p), plus the
// cross terms ah*bl + al*bh (the al*bl term, below 2^-48 relative, is dropped);
// an output row sum keeps a high float that takes every product's p through
// an exact two-sum and a low float that gathers all the low-order terms; the
// pair is renormalised once per output. The relative error of a row sum of T
// terms is about T * 2^-48 of the sum of the terms' magnitudes, against 2^-53
// for float64 -- far inside the 1e-12 amplitude bar. All float operations use
// the _rn intrinsics so that the compiler cannot contract a product and a sum
// into one FMA, which would break the error-free transformations.
//
// Conversions use integer instructions only: float64 -> (h, l) rounds the
// 52-bit significand to h's 24 bits (half up) and the signed remainder to l's
// 24 (48 bits kept, no bias towards zero; components below 2^-126 become 0);
// (h, l) -> float64 rebuilds each float as a float64 exactly from its bits and
// adds the two (one float64 add per component and pass).
//
// Scalar floats, one group per thread: packed pairs (add/sub/mul/fma.rn.f32x2,
// two groups per thread) measured slower here -- GB300 runs f32x2 FMAs at the
// same float rate as scalar ones (qgb_fma_probe: 80.2 vs 78.3 TFLOP/s), and
// the broadcast matrix pairs doubled the shared-memory loads.
#include <cstdlib>
#include <cstring>

#include "sweep_common.cuh"

namespace qgb {

struct dfc {  // one complex128 amplitude as two double-float numbers: 16 bytes, like double2
    float rh, rl, ih, il;
};

constexpr int kDfMaxK = 4;
constexpr int kDfMaxThreads = 512;
constexpr int kDfMatrixSlots = 256;  // one 4-qubit matrix of dfc

__device__ __forceinline__ void df_split(double x, float& h, float& l) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const uint32_t hw = uint32_t(b >> 32), lw = uint32_t(b);
    const uint32_t sign = hw & 0x80000000u;
    const int E = int((hw >> 20) & 0x7ffu);
    const int ef = E - 896;  // the float's biased exponent (1023 - 127 = 896)
    if (ef <= 0) {           // zero, and every |x| < 2^-126
        h = 0.f;
        l = 0.f;
        return;
    }
    // h: the significand rounded to 24 bits (half up); a carry out of the
    // significand moves into the exponent field, as it should
    const uint32_t up = (lw >> 28) & 1u;
    h = __uint_as_float(sign | (((uint32_t(ef) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29)) + up));
    // l = x - h: the 29 dropped bits (unit 2^(E - 1075)), less 2^29 when h was rounded up
    uint32_t r = lw & 0x1fffffffu;
    uint32_t lsign = sign;
    if (up) {
        r = 0x20000000u - r;
        lsign ^= 0x80000000u;
    }
    const int lz = __clz(r);
    const int el = E - lz - 917;  // biased exponent of r's leading bit: (31 - lz) + (E - 1075) + 127
    if (r == 0u || el <= 0) {
        l = 0.f;
        return;
    }
    uint32_t lb;
    if (lz >= 8) {
        lb = (uint32_t(el) << 23) | ((r << (lz - 8)) & 0x7fffffu);  // exact
    } else {  // leading bit to position 23, rounded half up (carry into the exponent field)
        const int sh = 8 - lz;
        lb = ((uint32_t(el) << 23) | ((r >> sh) & 0x7fffffu)) + ((r >> (sh - 1)) & 1u);
    }
    l = __uint_as_float(lsign | lb);
}

// A normal float (or zero) as a float64, exactly, from its bits; float
// subnormals (below 2^-126) become 0.
__device__ __forceinline__ double df_widen(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xffu;
    if (e == 0u) return 0.0;
    const uint32_t hw = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    return __hiloint2double(int(hw), int(b << 29));
}

__device__ __forceinline__ double df_join(float h, float l) { return df_widen(h) + df_widen(l); }

// (sh, sl) += (ah, al) * (bh, bl)
__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float t = __fadd_rn(sh, p);
    const float z = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z));
    sh = t;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// s = (re high, re low, im high, im low) += m * v
__device__ __forceinline__ void dfc_mac(float (&s)[4], const dfc& m, const dfc& v) {
    df_mac(s[0], s[1], m.rh, m.rl, v.rh, v.rl);
    df_mac(s[0], s[1], -m.ih, -m.il, v.ih, v.il);
    df_mac(s[2], s[3], m.rh, m.rl, v.ih, v.il);
    df_mac(s[2], s[3], m.ih, m.il, v.rh, v.rl);
}

__device__ __forceinline__ dfc dfc_finish(const float (&s)[4]) {
    dfc r;
    r.rh = __fadd_rn(s[0], s[1]);
    r.rl = __fsub_rn(s[1], __fsub_rn(r.rh, s[0]));
    r.ih = __fadd_rn(s[2], s[3]);
    r.il = __fsub_rn(s[3], __fsub_rn(r.ih, s[2]));
    return r;
}

// One dense op of width K on every group of a staged double-float tile; the
// op's matrix, already in double-float form, is in shared memory (msh).
template <int K>
__device__ __forceinline__ void tile_op_df(dfc* __restrict__ tile, int m, const int* pos_in,
                                           const dfc* __restrict__ msh, int tid, int nthr) {
    constexpr int D = 1 << K;
    int pos[K], srt[K];
#pragma unroll
    for (int j = 0; j < K; ++j) pos[j] = srt[j] = pos_in[j];
#pragma unroll
    for (int i = 1; i < K; ++i)
#pragma unroll
        for (int j = i; j > 0; --j)
            if (srt[j - 1] > srt[j]) {
                const int t = srt[j];
                srt[j] = srt[j - 1];
                srt[j - 1] = t;
            }
    uint32_t soff[D];
#pragma unroll
    for (int r = 0; r < D; ++r) {
        uint32_t o = 0;
#pragma unroll
        for (int j = 0; j < K; ++j) o |= uint32_t((r >> (K - 1 - j)) & 1) << pos[j];
        soff[r] = swz<double>(o);
    }
    const uint32_t groups = 1u << (m - K);
    for (uint32_t g = tid; g < groups; g += nthr) {
        uint32_t base = g;
#pragma unroll
        for (int j = 0; j < K; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
        const uint32_t sb = swz<double>(base);
        dfc v[D];
#pragma unroll
        for (int c = 0; c < D; ++c) v[c] = tile[sb ^ soff[c]];
#pragma unroll(K <= 2 ? D : 1)
        for (int r = 0; r < D; ++r) {
            float s[4] = {0.f, 0.f, 0.f, 0.f};
            const dfc* mrow = msh + r * D;
#pragma unroll
            for (int c = 0; c < D; ++c) dfc_mac(s, mrow[c], v[c]);
            uint32_t o = 0;
#pragma unroll
            for (int j = 0; j < K; ++j) o |= uint32_t((r >> (K - 1 - j)) & 1) << pos[j];
            tile[sb ^ swz<double>(o)] = dfc_finish(s);
        }
    }
}

template <int KMAX>
__global__ void __launch_bounds__(kDfMaxThreads) sweep_df_kernel(double2* __restrict__ sv,
                                                                 const double2* __restrict__ mats,
                                                                 const __grid_constant__ SweepArgs a, int nbuf) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = a.sw.low_bits, H = a.sw.n_high, m = L + H;
    // layout: nbuf tiles (2^m amplitudes of 16 bytes) | one op's matrix (<= 16 x 16) | hoff (2^H uint64)
    dfc* bufs = reinterpret_cast<dfc*>(smem_raw);
    dfc* msh = bufs + (size_t(nbuf) << m);  // one op's matrix
    uint64_t* hoff = reinterpret_cast<uint64_t*>(msh + kDfMatrixSlots);
    for (uint32_t h = threadIdx.x; h < (1u << H); h += blockDim.x) {
        uint64_t o = 0;
        for (int j = 0; j < H; ++j) o |= uint64_t((h >> j) & 1u) << a.sw.high_bits[j];
        hoff[h] = o;
    }
    __syncthreads();
    const uint32_t lmask = (1u << L) - 1;
    const uint64_t total = uint64_t(a.batch) * a.tiles;
    auto base_of = [&](uint64_t w) -> uint64_t {
        const uint64_t b = w / a.tiles, o = w - b * a.tiles;
        uint64_t base = uint64_t(b) * uint64_t(a.sv_stride);
        for (int j = 0; j < a.n_outer; ++j) base |= ((o >> j) & 1ull) << a.outer_bits[j];
        return base;
    };
    auto load_async = [&](uint64_t w, dfc* dst) {
        const uint64_t base = base_of(w);
        for (uint32_t e = threadIdx.x; e < (1u << m); e += blockDim.x)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                             uint32_t(__cvta_generic_to_shared(dst + swz<double>(e)))),
                         "l"(sv + (base + (hoff[e >> L] | (e & lmask))))
                         : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    uint64_t w = blockIdx.x;
    if (w < total) load_async(w, bufs);
    for (uint32_t i = 0; w < total; ++i, w += gridDim.x) {
        dfc* cur = bufs + (size_t(nbuf == 2 ? (i & 1) : 0) << m);
        const uint64_t wn = w + gridDim.x;
        if (nbuf == 2 && wn < total) {
            load_async(wn, bufs + (size_t((i + 1) & 1) << m));
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        // float64 -> double-float, in place (an elementwise map: the swizzle does not matter)
        for (uint32_t e = threadIdx.x; e < (1u << m); e += blockDim.x) {
            const double2 x = *reinterpret_cast<const double2*>(cur + e);
            dfc y;
            df_split(x.x, y.rh, y.rl);
            df_split(x.y, y.ih, y.il);
            cur[e] = y;
        }
        const double2* mb = mats + int64_t(w / a.tiles) * a.mat_stride;
        for (int op = 0; op < a.sw.n_ops; ++op) {
            const int k = a.sw.op_k[op];
            const int dd = 1 << (2 * k);
            const double2* mat = mb + a.sw.op_mat[op];
            __syncthreads();  // the previous op is done with msh (and, for op 0, the conversion with the tile)
            for (int e = threadIdx.x; e < dd; e += blockDim.x) {
                const double2 x = mat[e];
                dfc y;
                df_split(x.x, y.rh, y.rl);
                df_split(x.y, y.ih, y.il);
                msh[e] = y;
            }
            __syncthreads();
            const int* pos = a.sw.op_pos[op];
            if (k == 1) tile_op_df<1>(cur, m, pos, msh, threadIdx.x, blockDim.x);
            else if (k == 2) tile_op_df<2>(cur, m, pos, msh, threadIdx.x, blockDim.x);
            else if (k == 3) { if constexpr (KMAX >= 3) tile_op_df<3>(cur, m, pos, msh, threadIdx.x, blockDim.x); }
            else { if constexpr (KMAX >= 4) tile_op_df<4>(cur, m, pos, msh, threadIdx.x, blockDim.x); }
        }
        __syncthreads();
        const uint64_t base = base_of(w);
        for (uint32_t e = threadIdx.x; e < (1u << m); e += blockDim.x) {
            const dfc y = cur[swz<double>(e)];
            *reinterpret_cast<double2*>(sv + (base + (hoff[e >> L] | (e & lmask)))) =
                make_double2(df_join(y.rh, y.rl), df_join(y.ih, y.il));
        }
        __syncthreads();  // the buffer is free for the copy issued two tiles later
        if (nbuf == 1 && wn < total) load_async(wn, bufs);
    }
}

}  // namespace qgb

using namespace qgb;

namespace {

size_t df_smem_bytes(int m, int H, int kmax, int nbuf) {
    (void)kmax;
    return sizeof(dfc) * ((size_t(nbuf) << m) + kDfMatrixSlots) + sizeof(uint64_t) * (size_t(1) << H);
}

template <int KMAX>
int launch_df(void* sv, const void* mats, const SweepArgs& a, cudaStream_t st) {
    const int m = a.sw.low_bits + a.sw.n_high;
    auto kern = sweep_df_kernel<KMAX>;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
            return qgb_host::check_launch("double-float sweep attribute");
        attr = true;
    }
    for (int nbuf = 2; nbuf >= 1; --nbuf) {
        const size_t smem = df_smem_bytes(m, a.sw.n_high, KMAX, nbuf);
        if (smem > 227 * 1024) continue;
        int per_sm = 0, threads = 256;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem) != cudaSuccess)
            return qgb_host::check_launch("double-float sweep occupancy");
        if (per_sm < 1) continue;
        if (per_sm == 1) {
            int p512 = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p512, kern, 512, smem) != cudaSuccess)
                return qgb_host::check_launch("double-float sweep occupancy");
            if (p512 >= 1) threads = 512;
        }
        const uint64_t total = uint64_t(a.batch) * a.tiles;
        uint64_t grid = uint64_t(per_sm) * qgb_host::sm_count();
        if (grid > total) grid = total;
        kern<<<unsigned(grid), threads, smem, st>>>((double2*)sv, (const double2*)mats, a, nbuf);
        return qgb_host::check_launch("double-float sweep kernel");
    }
    return qgb_host::set_error(QGB_EINVAL, "sweep tile of 2^%d amplitudes does not fit in shared memory", m);
}

int g_c128_arith = -1;  // 0 = float64 kernels, 1 = double-float tile sweeps

}  // namespace

namespace qgb_host {

int c128_arith() {
    if (g_c128_arith < 0) {
        const char* e = getenv("QGB_C128_ARITH");
        g_c128_arith = (e && (strcmp(e, "fp64") == 0 || strcmp(e, "0") == 0)) ? 0 : 1;
    }
    return g_c128_arith;
}

int launch_sweep_df(void* sv, const void* mats, const qgb::SweepArgs& a, int kmax, cudaStream_t st) {
    switch (kmax) {
        case 1:
        case 2: return launch_df<2>(sv, mats, a, st);
        case 3: return launch_df<3>(sv, mats, a, st);
        case 4: return launch_df<4>(sv, mats, a, st);
    }
    return set_error(QGB_EINVAL, "double-float sweep op width %d unsupported (max %d)", kmax, kDfMaxK);
}

}  // namespace qgb_host

extern "C" int qgb_set_c128_arith(int mode) {
    if (mode != 0 && mode != 1)
        return qgb_host::set_error(QGB_EINVAL, "complex128 arithmetic %d unknown (0 = float64, 1 = double-float)", mode);
    g_c128_arith = mode;
    return QGB_OK;
}

extern "C" int qgb_get_c128_arith(void) { return qgb_host::c128_arith(); }
