// Measurement on the device: outcome probabilities of a subset of sites, shot
// sampling from them, and the post-measurement (collapsed) state.
//
// Replaces measure_sv and measure_and_collapse_sv (tensorQ/statevector_sim.py:
// 185-215): the reference forms the reduced density matrix of the measured
// sites on the host (rdm_from_sv, :182-183), samples its diagonal with
// numpy.random.choice and contracts a basis bra into the state.
//
//  * outcome_probs: p[b] = sum_r |psi(b, r)|^2, b the measured bits (site
//    list order, first site = most significant outcome bit), r the rest.
//    A warp sums one (bin, chunk of r) pair with lane-strided reads and a
//    fixed shuffle tree; a second kernel adds the chunks of each bin in
//    order. Float64 sums (complex64 states: float32 sums of 16 squares
//    folded into float64, the Acc rule), bitwise reproducible. When r has
//    fewer than 32 values one thread sums a bin.
//  * sample_outcomes: inclusive prefix sums of p in float64 (blocks of 4096,
//    the block totals scanned by one CTA, then offsets added), and per shot a
//    53-bit Philox uniform u scaled by the total and a binary search for the
//    first bin whose running sum exceeds it. Counter (shot lo, shot hi, 0, 1).
//  * collapse: out[j] = psi(outcome, j) / sqrt(p[outcome]), the unmeasured
//    sites keeping their order; the probability is read on the device.
#include <cstdio>

#include "philox.cuh"
#include "qgb_common.cuh"

namespace qgb {

constexpr int kMeasThreads = 256;
constexpr int kScanThreads = 1024;
constexpr int kScanChunk = 4 * kScanThreads;  // bins per scan block
constexpr int kMaxScanBlocks = 1 << 16;       // the block-total scan handles this many (2^28 bins)

struct ProbArgs {
    int n, m;
    int mbits[2 * QGB_MAX_QUBITS];  // flat bit of outcome bit i (i = 0: least significant)
    int sorted[2 * QGB_MAX_QUBITS];  // the same bits ascending
    uint64_t rest;                   // 2^(n - m)
    uint64_t chunks;                 // chunks of the rest per bin
    uint64_t chunk;                  // rest values per chunk
};

__device__ __forceinline__ uint64_t place_outcome(uint64_t b, const ProbArgs& a) {
    uint64_t o = 0;
    for (int i = 0; i < a.m; ++i) o |= ((b >> i) & 1ull) << a.mbits[i];
    return o;
}

template <typename T>
__global__ void __launch_bounds__(kMeasThreads) probs_warp_kernel(const cplx<T>* __restrict__ sv, double* __restrict__ part,
                                                                  const __grid_constant__ ProbArgs a) {
    const uint64_t w = (uint64_t(blockIdx.x) * kMeasThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint64_t bins = uint64_t(1) << a.m;
    if (w >= bins * a.chunks) return;  // whole warps leave together
    const uint64_t b = w % bins, c = w / bins;
    const uint64_t ob = place_outcome(b, a);
    Acc<T, 1> part_sum;
    for (uint64_t r = c * a.chunk + lane; r < (c + 1) * a.chunk; r += 32) {
        const cplx<T> v = sv[insert_zeros(r, a.sorted, a.m) | ob];
        part_sum.add(0, v.x * v.x + v.y * v.y);
        part_sum.step();
    }
    part_sum.flush();
    double acc = part_sum.d[0];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) part[c * bins + b] = acc;
}

template <typename T>
__global__ void __launch_bounds__(kMeasThreads) probs_thread_kernel(const cplx<T>* __restrict__ sv, double* __restrict__ probs,
                                                                    const __grid_constant__ ProbArgs a) {
    const uint64_t b = uint64_t(blockIdx.x) * kMeasThreads + threadIdx.x;
    if (b >= (uint64_t(1) << a.m)) return;
    const uint64_t ob = place_outcome(b, a);
    Acc<T, 1> acc;
    for (uint64_t r = 0; r < a.rest; ++r) {
        const cplx<T> v = sv[insert_zeros(r, a.sorted, a.m) | ob];
        acc.add(0, v.x * v.x + v.y * v.y);
        acc.step();
    }
    acc.flush();
    probs[b] = acc.d[0];
}

__global__ void __launch_bounds__(kMeasThreads) probs_finish_kernel(const double* __restrict__ part, double* __restrict__ probs,
                                                                    uint64_t bins, uint64_t chunks) {
    const uint64_t b = uint64_t(blockIdx.x) * kMeasThreads + threadIdx.x;
    if (b >= bins) return;
    double s = 0.0;
    for (uint64_t c = 0; c < chunks; ++c) s += part[c * bins + b];
    probs[b] = s;
}

// Inclusive scan of kScanChunk values per block (4 per thread, then a
// Hillis-Steele pass over the 1024 thread totals in shared memory).
__device__ __forceinline__ void block_scan_4(double v[4], double* sh, double& block_total) {
    v[1] += v[0];
    v[2] += v[1];
    v[3] += v[2];
    const int t = threadIdx.x;
    sh[t] = v[3];
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {
        const double add = t >= off ? sh[t - off] : 0.0;
        __syncthreads();
        sh[t] += add;
        __syncthreads();
    }
    const double before = t > 0 ? sh[t - 1] : 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] += before;
    block_total = sh[kScanThreads - 1];
    __syncthreads();
}

__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(const double* __restrict__ p, double* __restrict__ cdf,
                                                                   double* __restrict__ totals, uint64_t bins) {
    __shared__ double sh[kScanThreads];
    const uint64_t base = uint64_t(blockIdx.x) * kScanChunk + 4 * threadIdx.x;
    double v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = base + i < bins ? p[base + i] : 0.0;
    double tot;
    block_scan_4(v, sh, tot);
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (base + i < bins) cdf[base + i] = v[i];
    if (threadIdx.x == 0) totals[blockIdx.x] = tot;
}

// One CTA: exclusive offsets of up to kMaxScanBlocks block totals, in place
// (each thread scans a contiguous run serially, then the runs are offset).
__global__ void __launch_bounds__(kScanThreads) scan_totals_kernel(double* __restrict__ totals, int nblocks) {
    __shared__ double sh[kScanThreads];
    const int per = (nblocks + kScanThreads - 1) / kScanThreads;
    const int t = threadIdx.x, b0 = t * per;
    double run = 0.0;
    for (int i = 0; i < per && b0 + i < nblocks; ++i) run += totals[b0 + i];
    sh[t] = run;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {
        const double add = t >= off ? sh[t - off] : 0.0;
        __syncthreads();
        sh[t] += add;
        __syncthreads();
    }
    double acc = t > 0 ? sh[t - 1] : 0.0;
    for (int i = 0; i < per && b0 + i < nblocks; ++i) {
        const double x = totals[b0 + i];
        totals[b0 + i] = acc;
        acc += x;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_offset_kernel(double* __restrict__ cdf, const double* __restrict__ offs,
                                                                   uint64_t bins) {
    const uint64_t base = uint64_t(blockIdx.x) * kScanChunk;
    const double o = offs[blockIdx.x];
    for (int i = threadIdx.x; i < kScanChunk; i += kScanThreads)
        if (base + i < bins) cdf[base + i] += o;
}

__global__ void __launch_bounds__(kMeasThreads) sample_kernel(const double* __restrict__ cdf, uint64_t bins, int64_t shots,
                                                              uint32_t k0, uint32_t k1, int64_t* __restrict__ out) {
    const int64_t s = int64_t(blockIdx.x) * kMeasThreads + threadIdx.x;
    if (s >= shots) return;
    const double total = cdf[bins - 1];
    const double u = Philox::uniform4(uint32_t(uint64_t(s)), uint32_t(uint64_t(s) >> 32), 0u, 1u, k0, k1) * total;
    uint64_t lo = 0, hi = bins - 1;  // first bin with cdf > u (the last bin if rounding leaves none)
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (cdf[mid] > u)
            hi = mid;
        else
            lo = mid + 1;
    }
    out[s] = int64_t(lo);
}

template <typename T>
__global__ void __launch_bounds__(kMeasThreads) collapse_kernel(const cplx<T>* __restrict__ sv, cplx<T>* __restrict__ out,
                                                                const __grid_constant__ ProbArgs a, uint64_t outcome,
                                                                const double* __restrict__ probs) {
    const double p = probs[outcome];
    const T scale = T(1.0 / sqrt(p));
    const uint64_t ob = place_outcome(outcome, a);
    const uint64_t stride = uint64_t(gridDim.x) * kMeasThreads;
    for (uint64_t j = uint64_t(blockIdx.x) * kMeasThreads + threadIdx.x; j < a.rest; j += stride) {
        cplx<T> v = sv[insert_zeros(j, a.sorted, a.m) | ob];
        v.x *= scale;
        v.y *= scale;
        out[j] = v;
    }
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

namespace {

// Fills ProbArgs from the measured sites (outcome bit order = site order).
int prob_args(int n, const int* sites, int m, ProbArgs& a) {
    if (n < 1 || n > 2 * QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid", n);
    if (!sites) return set_error(QGB_EINVAL, "null site list");
    if (m < 1 || m > n) return set_error(QGB_EINVAL, "%d measured sites for n=%d", m, n);
    a = ProbArgs{};
    a.n = n;
    a.m = m;
    uint64_t seen = 0;
    for (int i = 0; i < m; ++i) {
        const int q = sites[i];
        if (q < 0 || q >= n) return set_error(QGB_EINVAL, "site %d out of range for n=%d", q, n);
        if (seen & (1ull << q)) return set_error(QGB_EINVAL, "site %d measured twice", q);
        seen |= 1ull << q;
        a.mbits[m - 1 - i] = n - 1 - q;  // sites[0] is the most significant outcome bit
    }
    for (int i = 0; i < m; ++i) a.sorted[i] = a.mbits[i];
    for (int i = 1; i < m; ++i)
        for (int j = i; j > 0 && a.sorted[j - 1] > a.sorted[j]; --j) {
            const int t = a.sorted[j];
            a.sorted[j] = a.sorted[j - 1];
            a.sorted[j - 1] = t;
        }
    a.rest = uint64_t(1) << (n - m);
    a.chunks = a.rest >= 32 ? (a.rest >= (uint64_t(1) << 12) ? a.rest >> 12 : 1) : 0;
    a.chunk = a.chunks ? a.rest / a.chunks : 0;
    return QGB_OK;
}

uint64_t probs_part_doubles(const ProbArgs& a) { return a.chunks ? a.chunks * (uint64_t(1) << a.m) : 0; }

}  // namespace

extern "C" size_t qgb_probs_scratch_bytes(int n, int m) {
    if (n < 1 || n > 2 * QGB_MAX_QUBITS || m < 1 || m > n) return 0;
    int sites[2 * QGB_MAX_QUBITS];
    for (int i = 0; i < m; ++i) sites[i] = i;
    ProbArgs a;
    if (prob_args(n, sites, m, a)) return 0;
    return size_t(probs_part_doubles(a)) * sizeof(double) + 256;
}

extern "C" int qgb_outcome_probs(const void* sv, int dtype, int n, const int* sites, int m, double* probs, void* scratch,
                                 size_t scratch_bytes, void* stream) {
    if (!sv || !probs) return set_error(QGB_EINVAL, "null pointer");
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    ProbArgs a;
    int rc = prob_args(n, sites, m, a);
    if (rc) return rc;
    if (m > 30) return set_error(QGB_EINVAL, "at most 30 measured sites (%d requested)", m);
    cudaStream_t st = (cudaStream_t)stream;
    const uint64_t bins = uint64_t(1) << m;
    if (a.chunks == 0) {
        const unsigned g = unsigned((bins + kMeasThreads - 1) / kMeasThreads);
        if (dtype == QGB_C64)
            probs_thread_kernel<float><<<g, kMeasThreads, 0, st>>>((const float2*)sv, probs, a);
        else
            probs_thread_kernel<double><<<g, kMeasThreads, 0, st>>>((const double2*)sv, probs, a);
        return check_launch("outcome probabilities");
    }
    const uint64_t need = probs_part_doubles(a) * sizeof(double);
    if (!scratch || scratch_bytes < need)
        return set_error(QGB_ESCRATCH, "scratch of %zu bytes needed (qgb_probs_scratch_bytes)", size_t(need) + 256);
    double* part = (double*)scratch;
    const uint64_t warps = bins * a.chunks;
    const uint64_t blocks = (warps * 32 + kMeasThreads - 1) / kMeasThreads;
    if (blocks > 0x7fffffffull) return set_error(QGB_EINVAL, "too many outcome bins");
    if (dtype == QGB_C64)
        probs_warp_kernel<float><<<unsigned(blocks), kMeasThreads, 0, st>>>((const float2*)sv, part, a);
    else
        probs_warp_kernel<double><<<unsigned(blocks), kMeasThreads, 0, st>>>((const double2*)sv, part, a);
    if ((rc = check_launch("outcome probabilities"))) return rc;
    probs_finish_kernel<<<unsigned((bins + kMeasThreads - 1) / kMeasThreads), kMeasThreads, 0, st>>>(part, probs, bins,
                                                                                                     a.chunks);
    return check_launch("outcome probabilities (finish)");
}

extern "C" size_t qgb_sample_scratch_bytes(int m) {
    if (m < 0 || m > 28) return 0;
    const uint64_t bins = uint64_t(1) << m;
    const uint64_t nb = (bins + kScanChunk - 1) / kScanChunk;
    return size_t((bins + nb) * sizeof(double)) + 256;
}

extern "C" int qgb_sample_outcomes(const double* probs, int m, int64_t shots, uint64_t seed, int64_t* out,
                                   void* scratch, size_t scratch_bytes, void* stream) {
    if (!probs || !out) return set_error(QGB_EINVAL, "null pointer");
    if (m < 0 || m > 28) return set_error(QGB_EINVAL, "sampling takes 0..28 outcome bits (%d requested)", m);
    if (shots < 1) return set_error(QGB_EINVAL, "shots must be positive");
    const uint64_t bins = uint64_t(1) << m;
    const uint64_t nb = (bins + kScanChunk - 1) / kScanChunk;
    if (nb > uint64_t(kMaxScanBlocks)) return set_error(QGB_EINVAL, "too many outcome bins to scan");
    if (!scratch || scratch_bytes < (bins + nb) * sizeof(double))
        return set_error(QGB_ESCRATCH, "scratch of %zu bytes needed (qgb_sample_scratch_bytes)",
                         qgb_sample_scratch_bytes(m));
    if (reinterpret_cast<uintptr_t>(scratch) % 8) return set_error(QGB_EINVAL, "misaligned scratch");
    double* cdf = (double*)scratch;
    double* totals = cdf + bins;
    cudaStream_t st = (cudaStream_t)stream;
    scan_blocks_kernel<<<unsigned(nb), kScanThreads, 0, st>>>(probs, cdf, totals, bins);
    int rc = check_launch("sample scan");
    if (rc) return rc;
    if (nb > 1) {
        scan_totals_kernel<<<1, kScanThreads, 0, st>>>(totals, int(nb));
        if ((rc = check_launch("sample scan totals"))) return rc;
        scan_offset_kernel<<<unsigned(nb), kScanThreads, 0, st>>>(cdf, totals, bins);
        if ((rc = check_launch("sample scan offsets"))) return rc;
    }
    const uint64_t g = (uint64_t(shots) + kMeasThreads - 1) / kMeasThreads;
    if (g > 0x7fffffffull) return set_error(QGB_EINVAL, "too many shots");
    sample_kernel<<<unsigned(g), kMeasThreads, 0, st>>>(cdf, bins, shots, uint32_t(seed), uint32_t(seed >> 32), out);
    return check_launch("sample outcomes");
}

extern "C" int qgb_collapse(const void* sv, int dtype, int n, const int* sites, int m, uint64_t outcome,
                            const double* probs, void* out, void* stream) {
    if (!sv || !out || !probs) return set_error(QGB_EINVAL, "null pointer");
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    ProbArgs a;
    const int rc = prob_args(n, sites, m, a);
    if (rc) return rc;
    if (m >= n) return set_error(QGB_EINVAL, "collapse keeps at least one site");
    if (m < 64 && outcome >= (uint64_t(1) << m)) return set_error(QGB_EINVAL, "outcome out of range");
    const uint64_t want = (a.rest + kMeasThreads - 1) / kMeasThreads;
    const unsigned g = unsigned(want < uint64_t(sm_count()) * 8 ? want : uint64_t(sm_count()) * 8);
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == QGB_C64)
        collapse_kernel<float><<<g, kMeasThreads, 0, st>>>((const float2*)sv, (float2*)out, a, outcome, probs);
    else
        collapse_kernel<double><<<g, kMeasThreads, 0, st>>>((const double2*)sv, (double2*)out, a, outcome, probs);
    return check_launch("collapse");
}
