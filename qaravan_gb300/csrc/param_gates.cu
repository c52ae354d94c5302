// Parametrised gate matrices for many parameter sets at once, and the chain
// rule from gate-matrix gradients to angle gradients, on the device.
//
// The reference builds every ParamGate matrix on the host with
// torch.linalg.matrix_exp(-i theta P) (core/param_gates.py:21-80; P a Pauli or
// Pauli pair, no factor 1/2) and copies it to the device per gate
// (tensorQ/statevector_sim.py:19-29). Since P^2 = I,
//     M(theta)    =  cos(theta) I - i sin(theta) P,
//     dM/dtheta   = -sin(theta) I - i cos(theta) P,
// so one thread per (parameter set, gate) writes M from the set's angle. The
// angle derivative of each gate comes from the rotation form of the adjoint
// step (2 Im <lam|P|phi>, equal to Re tr(G^H dM/dtheta) for the matrix
// gradient G); one thread per (set, parameter) then sums it over the gates
// that use the parameter, in the fixed order of a host-built CSR list.
// Kinds: 1 RX, 2 RY, 3 RZ (one site); 4 RXX, 5 RYY, 6 RZZ (two sites).
#include "qgb_common.cuh"

namespace qgb {

// Nonzero (row, col, value) entries of P: all Pauli products here have one
// nonzero per row, p[r] = column, ph[r] = value (+-1 or +-i).
__device__ __forceinline__ int pauli_perm(int kind, int r, double2& ph) {
    switch (kind) {
        case 1: ph = make_double2(1, 0); return r ^ 1;                                 // X
        case 2: ph = r == 0 ? make_double2(0, -1) : make_double2(0, 1); return r ^ 1;  // Y
        case 3: ph = make_double2(r == 0 ? 1 : -1, 0); return r;                       // Z
        case 4: ph = make_double2(1, 0); return r ^ 3;                                 // XX
        case 5: ph = make_double2((r == 0 || r == 3) ? -1 : 1, 0); return r ^ 3;       // YY: (Y x Y)[r][r ^ 3]
        default: ph = make_double2((r == 0 || r == 3) ? 1 : -1, 0); return r;          // ZZ
    }
}

__device__ __forceinline__ int kind_dim(int kind) { return kind <= 3 ? 2 : 4; }

template <typename T>
__global__ void param_matrices_kernel(const int* __restrict__ kinds, const int* __restrict__ pidx, int ngates,
                                      const double* __restrict__ params, int nparams, int64_t nsets,
                                      cplx<T>* __restrict__ out, int64_t gate_stride, int64_t set_stride) {
    const int64_t item = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (item >= nsets * ngates) return;
    const int64_t s = item / ngates;
    const int g = int(item - s * ngates);
    const int kind = kinds[g];
    if (kind < 1 || kind > 6) return;  // a fixed gate: its matrix is the caller's
    const int d = kind_dim(kind);
    const double th = params[s * nparams + pidx[g]];
    double sn, cs;
    sincos(th, &sn, &cs);
    cplx<T>* m = out + s * set_stride + int64_t(g) * gate_stride;
    for (int i = 0; i < d * d; ++i) m[i] = mk<T>(T(0), T(0));
    for (int r = 0; r < d; ++r) {
        double2 ph;
        const int c = pauli_perm(kind, r, ph);
        // -i sin(theta) * ph at (r, c); cos(theta) on the diagonal
        double re = sn * ph.y, im = -sn * ph.x;
        if (c == r) re += cs;
        m[r * d + c] = mk<T>(T(re), T(im));
        if (c != r) m[r * d + r] = mk<T>(T(cs), T(0));
    }
}

// grad_out[s * nparams + j] = scale * sum over the gates g of parameter j
// (CSR: csr_gate[csr_ptr[j] .. csr_ptr[j+1]), in that order) of
// gate_values[g * nsets + s] -- per-gate angle derivatives, e.g. the rotation
// form of the adjoint step, Im <lam|P|phi>, for which scale = 2.
__global__ void param_grads_kernel(const int* __restrict__ csr_ptr, const int* __restrict__ csr_gate, int nparams,
                                   int64_t nsets, const double* __restrict__ gate_values, double scale,
                                   double* __restrict__ grad_out) {
    const int64_t item = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (item >= nsets * nparams) return;
    const int64_t s = item / nparams;
    const int j = int(item - s * nparams);
    double acc = 0.0;
    for (int e = csr_ptr[j]; e < csr_ptr[j + 1]; ++e) acc += gate_values[int64_t(csr_gate[e]) * nsets + s];
    grad_out[s * nparams + j] = scale * acc;
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

extern "C" int qgb_param_matrices(const int* kinds, const int* pidx, int ngates, const double* params, int nparams,
                                  int64_t nsets, void* out, int dtype, int64_t gate_stride, int64_t set_stride,
                                  void* stream) {
    if (!kinds || !pidx || !params || !out) return set_error(QGB_EINVAL, "null pointer");
    if (ngates < 1 || nparams < 1 || nsets < 1) return set_error(QGB_EINVAL, "empty parameter batch");
    if (gate_stride < 16 || set_stride < gate_stride * ngates)
        return set_error(QGB_EINVAL, "strides too small for 4x4 matrices");
    const int64_t items = nsets * ngates;
    const unsigned g = unsigned((items + 255) / 256);
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == QGB_C64)
        param_matrices_kernel<float><<<g, 256, 0, st>>>(kinds, pidx, ngates, params, nparams, nsets, (float2*)out,
                                                        gate_stride, set_stride);
    else if (dtype == QGB_C128)
        param_matrices_kernel<double><<<g, 256, 0, st>>>(kinds, pidx, ngates, params, nparams, nsets, (double2*)out,
                                                         gate_stride, set_stride);
    else
        return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    return check_launch("param matrices");
}

extern "C" int qgb_param_grads(const int* csr_ptr, const int* csr_gate, int nparams, int64_t nsets,
                               const double* gate_values, double scale, double* grad_out, void* stream) {
    if (!csr_ptr || !csr_gate || !gate_values || !grad_out) return set_error(QGB_EINVAL, "null pointer");
    if (nparams < 1 || nsets < 1) return set_error(QGB_EINVAL, "empty parameter batch");
    const int64_t items = nsets * nparams;
    const unsigned g = unsigned((items + 255) / 256);
    param_grads_kernel<<<g, 256, 0, (cudaStream_t)stream>>>(csr_ptr, csr_gate, nparams, nsets, gate_values, scale,
                                                            grad_out);
    return check_launch("param grads");
}
