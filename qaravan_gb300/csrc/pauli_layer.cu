// One Pauli string per state, applied in place to a batch of states: the
// sampled noise layers of Monte-Carlo trajectories.
//
// The reference's MonteCarloSim (tensorQ/monte_carlo_sim.py:14-28) turns each
// sampled Pauli string into single-qubit X/Y/Z gates (pauli_string_to_gates,
// core/gates.py:304-305) and runs them through a fresh StatevectorSim per
// sample. Here state b gets P_b = i^{ny_b} X^{x_b} Z^{z_b} (flat-bit masks,
// Y sites in both masks):
//     psi'[i] = i^{ny} (-1)^{popcount((i ^ x) & z)} psi[i ^ x],
// one read and one write of each state (pairs i, i ^ x swap within a thread).
#include "qgb_common.cuh"

namespace qgb {

template <typename T>
__device__ __forceinline__ cplx<T> times_phase(cplx<T> v, int k, bool neg) {
    // v * i^k * (neg ? -1 : 1)
    cplx<T> r = v;
    if (k & 1) r = mk<T>(-v.y, v.x);
    if (k & 2) r = mk<T>(-r.x, -r.y);
    if (neg) r = mk<T>(-r.x, -r.y);
    return r;
}

template <typename T>
__global__ void __launch_bounds__(256) pauli_layer_kernel(cplx<T>* __restrict__ sv, int n, const uint64_t* __restrict__ xm,
                                                          const uint64_t* __restrict__ zm, const int* __restrict__ ny,
                                                          int64_t stride) {
    const int64_t b = blockIdx.y;
    const uint64_t x = xm[b], z = zm[b];
    const int k = ny[b] & 3;
    const uint64_t len = uint64_t(1) << n, mask = len - 1;
    if (((x | z) & ~mask) != 0) return;  // masks beyond the state's bits (rejected on the host too)
    cplx<T>* s = sv + b * stride;
    const uint64_t step = uint64_t(gridDim.x) * blockDim.x;
    if (x == 0) {
        if (z == 0 && k == 0) return;
        for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < len; i += step)
            s[i] = times_phase<T>(s[i], k, __popcll(i & z) & 1);
        return;
    }
    const int hb = 63 - __clzll(x);  // the pair (i, i ^ x) has bit hb clear in i
    for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < (len >> 1); g += step) {
        const uint64_t i = ((g >> hb) << (hb + 1)) | (g & ((uint64_t(1) << hb) - 1));
        const uint64_t j = i ^ x;
        const cplx<T> a = s[i], c = s[j];
        s[i] = times_phase<T>(c, k, __popcll(j & z) & 1);  // psi'[i] from psi[j], j = i ^ x
        s[j] = times_phase<T>(a, k, __popcll(i & z) & 1);
    }
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

extern "C" int qgb_pauli_layer(void* sv, int dtype, int n, const uint64_t* xmask, const uint64_t* zmask, const int* ny,
                               int64_t batch, int64_t sv_stride, void* stream) {
    if (!sv || !xmask || !zmask || !ny) return set_error(QGB_EINVAL, "null pointer");
    if (n < 1 || n > 2 * QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid", n);
    if (batch < 1 || batch > 65535) return set_error(QGB_EINVAL, "batch %lld not in [1, 65535]", (long long)batch);
    if (batch > 1 && sv_stride < (int64_t(1) << n)) return set_error(QGB_EINVAL, "state stride smaller than the state");
    const uint64_t half = uint64_t(1) << (n - 1);
    uint64_t per = uint64_t(sm_count()) * 8 / uint64_t(batch);
    if (per < 1) per = 1;
    const uint64_t need = (half + 255) / 256;
    dim3 grid(unsigned(need < per ? need : per), unsigned(batch));
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == QGB_C64)
        pauli_layer_kernel<float><<<grid, 256, 0, st>>>((float2*)sv, n, xmask, zmask, ny, sv_stride);
    else if (dtype == QGB_C128)
        pauli_layer_kernel<double><<<grid, 256, 0, st>>>((double2*)sv, n, xmask, zmask, ny, sv_stride);
    else
        return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    return check_launch("pauli layer");
}
