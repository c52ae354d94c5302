// Dense k-local gate application straight on HBM (one read + one write of the
// state per gate), basis-state initialisation and per-state scaling.
//
// Replaces the reference's per-gate `op_action` (tensorQ/statevector_sim.py:124-140):
// where the reference permutes the state, runs a tensordot and permutes back
// (2-3 passes over HBM per gate), this is a single coalesced pass.
//
//  * dense_reg_kernel<T, K>, K <= 4: one thread owns one group of 2^K partner
//    amplitudes in registers; the matrix is staged in shared memory (in
//    registers for K <= 2).
//  * dense_smem_kernel<T, K>, K = 5, 6: a CTA stages 1024 amplitudes and the
//    transposed matrix in shared memory and forms the 2^K x G product with
//    one output row per thread (conflict-free matrix reads, broadcast state
//    reads).
#include <cstdio>

#include "qgb_common.cuh"

namespace qgb {

struct DenseArgs {
    int n, k;
    int sorted[QGB_MAX_K];
    uint64_t off_in[1 << QGB_MAX_K];
    uint64_t off_out[1 << QGB_MAX_K];
    int64_t op_stride, batch, sv_stride;
    uint64_t groups;
};

template <typename T, int K>
__global__ void __launch_bounds__(256) dense_reg_kernel(cplx<T>* __restrict__ sv, const cplx<T>* __restrict__ op,
                                                        const __grid_constant__ DenseArgs a) {
    constexpr int D = 1 << K;
    using C = cplx<T>;
    __shared__ __align__(16) C M[D * D];
    const int64_t b = blockIdx.y;
    const C* opb = op + b * a.op_stride;
    for (int i = threadIdx.x; i < D * D; i += blockDim.x) M[i] = opb[i];
    __syncthreads();
    C* s = sv + b * a.sv_stride;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    if constexpr (K <= 2) {
        C m[D * D];
#pragma unroll
        for (int i = 0; i < D * D; ++i) m[i] = M[i];
        for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < a.groups; g += stride) {
            const uint64_t base = insert_zeros(g, a.sorted, K);
            C v[D];
#pragma unroll
            for (int c = 0; c < D; ++c) v[c] = s[base + a.off_in[c]];
#pragma unroll
            for (int r = 0; r < D; ++r) {
                C acc = mk<T>(0, 0);
#pragma unroll
                for (int c = 0; c < D; ++c) cfma(acc, m[r * D + c], v[c]);
                s[base + a.off_out[r]] = acc;
            }
        }
    } else if (sizeof(T) == 4 && a.groups >= 2) {
        // complex64, K = 3, 4: each thread takes groups g and g + groups/2 together so that
        // every matrix element (two per 16-byte shared-memory load) feeds two groups
        const uint64_t half = a.groups >> 1;
        for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < half; g += stride) {
            const uint64_t b0 = insert_zeros(g, a.sorted, K), b1 = insert_zeros(g + half, a.sorted, K);
            C v0[D], v1[D];
#pragma unroll
            for (int c = 0; c < D; ++c) {
                v0[c] = s[b0 + a.off_in[c]];
                v1[c] = s[b1 + a.off_in[c]];
            }
#pragma unroll 1
            for (int r = 0; r < D; ++r) {
                const float4* m4 = reinterpret_cast<const float4*>(M + r * D);
                C a0 = mk<T>(0, 0), a1 = mk<T>(0, 0);
#pragma unroll
                for (int c = 0; c < D; c += 2) {
                    const float4 q = m4[c >> 1];
                    const C e0 = mk<T>(T(q.x), T(q.y)), e1 = mk<T>(T(q.z), T(q.w));
                    cfma(a0, e0, v0[c]);
                    cfma(a1, e0, v1[c]);
                    cfma(a0, e1, v0[c + 1]);
                    cfma(a1, e1, v1[c + 1]);
                }
                s[b0 + a.off_out[r]] = a0;
                s[b1 + a.off_out[r]] = a1;
            }
        }
    } else {
        for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < a.groups; g += stride) {
            const uint64_t base = insert_zeros(g, a.sorted, K);
            C v[D];
#pragma unroll
            for (int c = 0; c < D; ++c) v[c] = s[base + a.off_in[c]];
#pragma unroll 1
            for (int r = 0; r < D; ++r) {
                const C* mrow = M + r * D;
                C acc = mk<T>(0, 0);
#pragma unroll
                for (int c = 0; c < D; ++c) cfma(acc, mrow[c], v[c]);
                s[base + a.off_out[r]] = acc;
            }
        }
    }
}

template <typename T, int K> struct SmemGeom {
    static constexpr int D = 1 << K;
    static constexpr int G = 1024 / D;      // groups per chunk
    static constexpr int NG = 256 / D;      // group slots across the CTA
    static constexpr int PER = G / NG;      // groups per thread
    static constexpr size_t bytes = sizeof(cplx<T>) * (size_t(D) * D + size_t(G) * D);
};

template <typename T, int K>
__global__ void __launch_bounds__(256) dense_smem_kernel(cplx<T>* __restrict__ sv, const cplx<T>* __restrict__ op,
                                                         const __grid_constant__ DenseArgs a) {
    using Geo = SmemGeom<T, K>;
    constexpr int D = Geo::D, G = Geo::G, NG = Geo::NG, PER = Geo::PER;
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* MT = reinterpret_cast<C*>(smem_raw);  // MT[c * D + r] = M[r][c]
    C* V = MT + D * D;                       // V[gi * D + c]
    const int64_t b = blockIdx.y;
    const C* opb = op + b * a.op_stride;
    for (int i = threadIdx.x; i < D * D; i += blockDim.x) {
        const int r = i / D, c = i % D;
        MT[c * D + r] = opb[i];
    }
    C* s = sv + b * a.sv_stride;
    const int r = threadIdx.x % D, gs = threadIdx.x / D;
    const uint64_t nchunks = (a.groups + G - 1) / G;  // the last chunk may be partial (small vectors)
    __syncthreads();
    for (uint64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const uint64_t g0 = ch * G;
        for (int i = threadIdx.x; i < G * D; i += blockDim.x) {
            const int gi = i / D, c = i % D;
            V[i] = (g0 + gi < a.groups) ? s[insert_zeros(g0 + gi, a.sorted, K) + a.off_in[c]] : mk<T>(0, 0);
        }
        __syncthreads();
        C acc[PER];
#pragma unroll
        for (int j = 0; j < PER; ++j) acc[j] = mk<T>(0, 0);
#pragma unroll 4
        for (int c = 0; c < D; ++c) {
            const C m = MT[c * D + r];
#pragma unroll
            for (int j = 0; j < PER; ++j) cfma(acc[j], m, V[(gs + j * NG) * D + c]);
        }
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int gi = gs + j * NG;
            if (g0 + gi < a.groups) s[insert_zeros(g0 + gi, a.sorted, K) + a.off_out[r]] = acc[j];
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void init_basis_kernel(cplx<T>* __restrict__ sv, uint64_t len, uint64_t index, int64_t sv_stride) {
    cplx<T>* s = sv + int64_t(blockIdx.y) * sv_stride;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < len; i += stride)
        s[i] = mk<T>(i == index ? T(1) : T(0), T(0));
}

template <typename T>
__global__ void scale_kernel(cplx<T>* __restrict__ sv, uint64_t len, const double* __restrict__ scale,
                             int64_t sv_stride) {
    cplx<T>* s = sv + int64_t(blockIdx.y) * sv_stride;
    const T f = T(scale[blockIdx.y]);
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < len; i += stride) {
        cplx<T> v = s[i];
        v.x *= f;
        v.y *= f;
        s[i] = v;
    }
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

namespace {

unsigned grid_x_for(uint64_t work, int64_t batch, unsigned threads) {
    const uint64_t target = uint64_t(sm_count()) * 8;
    uint64_t per_state = (target + uint64_t(batch) - 1) / uint64_t(batch);
    if (per_state < 1) per_state = 1;
    uint64_t need = (work + threads - 1) / threads;
    if (need < 1) need = 1;
    return unsigned(need < per_state ? need : per_state);
}

template <typename T, int K>
int launch_dense(void* sv, const void* op, const DenseArgs& a, cudaStream_t st) {
    if constexpr (K <= 4) {
        dim3 grid(grid_x_for(a.groups, a.batch, 256), unsigned(a.batch));
        dense_reg_kernel<T, K><<<grid, 256, 0, st>>>((cplx<T>*)sv, (const cplx<T>*)op, a);
    } else {
        using Geo = SmemGeom<T, K>;
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(dense_smem_kernel<T, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(Geo::bytes)) != cudaSuccess)
                return check_launch("dense_smem attribute");
            attr = true;
        }
        const uint64_t nchunks = (a.groups + Geo::G - 1) / Geo::G;
        dim3 grid(grid_x_for(nchunks * 256, a.batch, 256), unsigned(a.batch));
        dense_smem_kernel<T, K><<<grid, 256, Geo::bytes, st>>>((cplx<T>*)sv, (const cplx<T>*)op, a);
    }
    return check_launch("dense gate kernel");
}

template <typename T>
int dispatch_dense(void* sv, const void* op, const DenseArgs& a, cudaStream_t st) {
    switch (a.k) {
        case 1: return launch_dense<T, 1>(sv, op, a, st);
        case 2: return launch_dense<T, 2>(sv, op, a, st);
        case 3: return launch_dense<T, 3>(sv, op, a, st);
        case 4: return launch_dense<T, 4>(sv, op, a, st);
        case 5: return launch_dense<T, 5>(sv, op, a, st);
        case 6: return launch_dense<T, 6>(sv, op, a, st);
    }
    return set_error(QGB_EINVAL, "k=%d out of range", a.k);
}

}  // namespace

namespace qgb_host {

// Applies a dense 2^k x 2^k op whose input bit j is in_bits[j] and output bit
// j is out_bits[j] (same set of bits) to `batch` vectors of 2^nbits entries.
int apply_dense_bits(void* sv, int dtype, int nbits, const int* in_bits, const int* out_bits, int k,
                     const void* op, int64_t op_stride, int64_t batch, int64_t sv_stride, cudaStream_t st,
                     int unitary = 0, double* chain = nullptr, int link = 0, const double* scale = nullptr) {
    if (!sv || !op) return set_error(QGB_EINVAL, "null state or operator pointer");
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    if (k < 1 || k > QGB_MAX_K) return set_error(QGB_EINVAL, "gate width k=%d not in [1, %d]", k, QGB_MAX_K);
    if (nbits < k || nbits > 2 * QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid for k=%d", nbits, k);
    if (batch < 1 || batch > 65535) return set_error(QGB_EINVAL, "batch %lld not in [1, 65535]", (long long)batch);
    if (batch > 1 && sv_stride < (int64_t(1) << nbits))
        return set_error(QGB_EINVAL, "state stride %lld smaller than the state", (long long)sv_stride);
    if (op_stride < 0) return set_error(QGB_EINVAL, "negative operator stride");
    const uintptr_t esz = dtype == QGB_C64 ? 8 : 16;
    if ((reinterpret_cast<uintptr_t>(sv) % esz) || (reinterpret_cast<uintptr_t>(op) % esz))
        return set_error(QGB_EINVAL, "state or operator pointer not aligned to the element size");
    DenseArgs a{};
    a.n = nbits;
    a.k = k;
    uint64_t seen = 0;
    for (int j = 0; j < k; ++j) {
        if (in_bits[j] < 0 || in_bits[j] >= nbits) return set_error(QGB_EINVAL, "target bit %d out of range", in_bits[j]);
        if (seen & (1ull << in_bits[j])) return set_error(QGB_EINVAL, "repeated target bit %d", in_bits[j]);
        seen |= 1ull << in_bits[j];
        a.sorted[j] = in_bits[j];
    }
    uint64_t seen_out = 0;
    for (int j = 0; j < k; ++j) seen_out |= 1ull << out_bits[j];
    if (seen_out != seen) return set_error(QGB_EINVAL, "output bits are not a permutation of the input bits");
    for (int i = 1; i < k; ++i)
        for (int j = i; j > 0 && a.sorted[j - 1] > a.sorted[j]; --j) {
            int t = a.sorted[j];
            a.sorted[j] = a.sorted[j - 1];
            a.sorted[j - 1] = t;
        }
    for (int r = 0; r < (1 << k); ++r) {
        a.off_in[r] = matrix_offset(r, in_bits, k);
        a.off_out[r] = matrix_offset(r, out_bits, k);
    }
    a.op_stride = op_stride;
    a.batch = batch;
    a.sv_stride = sv_stride;
    a.groups = uint64_t(1) << (nbits - k);
    if (unitary == 2) {
        if (dtype == QGB_C64) {
            const int rc = try_dense_tc(sv, op, nbits, a.sorted, in_bits, out_bits, k, op_stride, batch, sv_stride, 2,
                                        st, chain, link);
            if (rc != QGB_EDECLINE) return rc;
        }
        // not on the chain kernel: clear the chain, so that the next pass starts a new one
        if (cudaMemsetAsync(chain, 0, 6 * sizeof(double), st) != cudaSuccess) return check_launch("norm chain reset");
        unitary = 1;
    }
    if (dtype == QGB_C64) {
        const int rc = try_dense_tc(sv, op, nbits, a.sorted, in_bits, out_bits, k, op_stride, batch, sv_stride,
                                    unitary, st, nullptr, 0, scale);
        if (rc != QGB_EDECLINE) return rc;
    }
    const int rc = dtype == QGB_C64 ? dispatch_dense<float>(sv, op, a, st) : dispatch_dense<double>(sv, op, a, st);
    if (rc || !scale) return rc;
    // the CUDA-core kernels take no factor: one more pass multiplies the result by it
    return qgb_scale(sv, dtype, nbits, scale, 1, 0, st);
}

}  // namespace qgb_host

namespace {

int op_action(void* sv, int dtype, int n, const int* indices, int k, const void* op, int64_t op_stride,
              int64_t batch, int64_t sv_stride, void* stream, int unitary, double* chain = nullptr, int link = 0) {
    if (n < 1 || n > QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d not in [1, %d]", n, QGB_MAX_QUBITS);
    if (!indices) return set_error(QGB_EINVAL, "null indices");
    if (k < 1 || k > QGB_MAX_K) return set_error(QGB_EINVAL, "gate width k=%d not in [1, %d]", k, QGB_MAX_K);
    int bits[QGB_MAX_K];
    for (int j = 0; j < k; ++j) {
        if (indices[j] < 0 || indices[j] >= n) return set_error(QGB_EINVAL, "site %d out of range for n=%d", indices[j], n);
        bits[j] = n - 1 - indices[j];
    }
    return apply_dense_bits(sv, dtype, n, bits, bits, k, op, op_stride, batch, sv_stride, (cudaStream_t)stream,
                            unitary, chain, link);
}

}  // namespace

extern "C" int qgb_op_action(void* sv, int dtype, int n, const int* indices, int k, const void* op,
                             int64_t op_stride, int64_t batch, int64_t sv_stride, void* stream) {
    return op_action(sv, dtype, n, indices, k, op, op_stride, batch, sv_stride, stream, 0);
}

extern "C" int qgb_op_action_unitary(void* sv, int dtype, int n, const int* indices, int k, const void* op,
                                     int64_t op_stride, int64_t batch, int64_t sv_stride, void* stream) {
    return op_action(sv, dtype, n, indices, k, op, op_stride, batch, sv_stride, stream, 1);
}

extern "C" int qgb_op_action_unitary_chain(void* sv, int dtype, int n, const int* indices, int k, const void* op,
                                           int64_t op_stride, int64_t batch, int64_t sv_stride, double* chain,
                                           int link, void* stream) {
    if (!chain || (reinterpret_cast<uintptr_t>(chain) % sizeof(double)))
        return set_error(QGB_EINVAL, "norm chain buffer missing or not 8-byte aligned");
    if (link < 0) return set_error(QGB_EINVAL, "negative chain link %d", link);
    return op_action(sv, dtype, n, indices, k, op, op_stride, batch, sv_stride, stream, 2, chain, link);
}

extern "C" int qgb_op_action_scaled(void* sv, int dtype, int n, const int* indices, int k, const void* op,
                                    const double* factor, void* stream) {
    if (!factor || (reinterpret_cast<uintptr_t>(factor) % sizeof(double)))
        return set_error(QGB_EINVAL, "factor missing or not 8-byte aligned");
    if (n < 1 || n > QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d not in [1, %d]", n, QGB_MAX_QUBITS);
    if (!indices) return set_error(QGB_EINVAL, "null indices");
    if (k < 1 || k > QGB_MAX_K) return set_error(QGB_EINVAL, "gate width k=%d not in [1, %d]", k, QGB_MAX_K);
    int bits[QGB_MAX_K];
    for (int j = 0; j < k; ++j) {
        if (indices[j] < 0 || indices[j] >= n) return set_error(QGB_EINVAL, "site %d out of range for n=%d", indices[j], n);
        bits[j] = n - 1 - indices[j];
    }
    return apply_dense_bits(sv, dtype, n, bits, bits, k, op, 0, 1, 0, (cudaStream_t)stream, 0, nullptr, 0, factor);
}

extern "C" int qgb_dm_apply_superop(void* rho, int dtype, int n, const int* indices, int k, const void* superop,
                                    int64_t batch, int64_t rho_stride, void* stream) {
    if (n < 1 || 2 * n > 2 * QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid", n);
    if (!indices) return set_error(QGB_EINVAL, "null indices");
    if (k < 1 || 2 * k > QGB_MAX_K) return set_error(QGB_EINVAL, "superoperator on k=%d sites unsupported", k);
    int sorted_sites[QGB_MAX_K];
    for (int j = 0; j < k; ++j) {
        if (indices[j] < 0 || indices[j] >= n) return set_error(QGB_EINVAL, "site %d out of range for n=%d", indices[j], n);
        sorted_sites[j] = indices[j];
    }
    for (int i = 1; i < k; ++i)
        for (int j = i; j > 0 && sorted_sites[j - 1] > sorted_sites[j]; --j) {
            int t = sorted_sites[j];
            sorted_sites[j] = sorted_sites[j - 1];
            sorted_sites[j - 1] = t;
        }
    // vec(rho): ket site q -> bit 2n-1-q, bra site q -> bit n-1-q. Superop row/col
    // bits: (bra legs.., ket legs..); inputs in `indices` order, outputs ascending.
    int in_bits[QGB_MAX_K], out_bits[QGB_MAX_K];
    for (int j = 0; j < k; ++j) {
        in_bits[j] = n - 1 - indices[j];
        in_bits[k + j] = 2 * n - 1 - indices[j];
        out_bits[j] = n - 1 - sorted_sites[j];
        out_bits[k + j] = 2 * n - 1 - sorted_sites[j];
    }
    return apply_dense_bits(rho, dtype, 2 * n, in_bits, out_bits, 2 * k, superop, 0, batch, rho_stride,
                            (cudaStream_t)stream);
}

extern "C" int qgb_init_basis(void* sv, int dtype, int n, uint64_t index, int64_t batch, int64_t sv_stride,
                              void* stream) {
    if (!sv) return set_error(QGB_EINVAL, "null state");
    if (n < 1 || n > 2 * QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid", n);
    if (index >= (uint64_t(1) << n)) return set_error(QGB_EINVAL, "basis index out of range");
    if (batch < 1 || batch > 65535) return set_error(QGB_EINVAL, "batch out of range");
    const uint64_t len = uint64_t(1) << n;
    dim3 grid(grid_x_for(len, batch, 256), unsigned(batch));
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == QGB_C64)
        init_basis_kernel<float><<<grid, 256, 0, st>>>((float2*)sv, len, index, sv_stride);
    else if (dtype == QGB_C128)
        init_basis_kernel<double><<<grid, 256, 0, st>>>((double2*)sv, len, index, sv_stride);
    else
        return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    return check_launch("init_basis");
}

extern "C" int qgb_scale(void* sv, int dtype, int n, const double* scale, int64_t batch, int64_t sv_stride,
                         void* stream) {
    if (!sv || !scale) return set_error(QGB_EINVAL, "null pointer");
    if (n < 1 || n > 2 * QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid", n);
    if (batch < 1 || batch > 65535) return set_error(QGB_EINVAL, "batch out of range");
    const uint64_t len = uint64_t(1) << n;
    dim3 grid(grid_x_for(len, batch, 256), unsigned(batch));
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == QGB_C64)
        scale_kernel<float><<<grid, 256, 0, st>>>((float2*)sv, len, scale, sv_stride);
    else if (dtype == QGB_C128)
        scale_kernel<double><<<grid, 256, 0, st>>>((double2*)sv, len, scale, sv_stride);
    else
        return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    return check_launch("scale");
}
