// Expectation values and other reductions, accumulated in float64.
//
// Replaces the reference's ncon-based reductions (pauli_expectation_sv,
// tensorQ/statevector_sim.py:217-234; local/one_local_expectation :63-94;
// partial_overlap :155-180; DensityMatrixSim expectations and trace,
// tensorQ/density_matrix_sim.py:49-89). Each reduction reads the state once
// per group of terms, keeps per-thread float64 sums (complex64 states: float32
// chunk sums folded into float64, see Acc), reduces a block in a fixed
// shuffle order, writes one partial per block into caller-provided scratch,
// and a second kernel sums the partials in a fixed order, so the result is
// bitwise reproducible run to run.
#include <cstring>
#include <vector>

#include "qgb_common.cuh"

namespace qgb {

constexpr int kRedThreads = 256;

// Blocks per vector for a reduction over 2^nbits entries (independent of the
// device, so the scratch size is a pure function of the problem).
__host__ __device__ inline int red_blocks(int nbits) {
    const int64_t len = int64_t(1) << nbits;
    int64_t b = len / 4096;
    if (b < 1) b = 1;
    if (b > 1216) b = 1216;
    return int(b);
}

template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double* __restrict__ dst, int64_t dst_stride,
                                                   int nvalid = NV) {
    __shared__ double red[kRedThreads / 32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        double x = v[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][j] = x;
    }
    __syncthreads();
    if (threadIdx.x < nvalid) {
        double s = 0;
        for (int w = 0; w < kRedThreads / 32; ++w) s += red[w][threadIdx.x];
        dst[int64_t(threadIdx.x) * dst_stride] = s;
    }
    __syncthreads();
}

struct PauliGroup {
    uint64_t xmask;
    int nterms;
    int slot0;  // first output slot of this group
    uint64_t zmask[32];
    int ny[32];
    double coeff[32];
};

// Re( i^ny * z )
template <typename R>
__device__ __forceinline__ R re_iny(R re, R im, int ny) {
    switch (ny & 3) {
        case 0: return re;
        case 1: return -im;
        case 2: return -re;
        default: return im;
    }
}

// One pass over the vector for all terms sharing one X mask.
// partials[(b * nslots + slot) * nblk + blk]
__device__ __forceinline__ int popc_any(uint32_t v) { return __popc(v); }
__device__ __forceinline__ int popc_any(uint64_t v) { return __popcll(v); }

// I: the index type, 32-bit for vectors of up to 2^31 entries (cheaper loop and
// mask arithmetic than 64-bit), else 64-bit.
template <typename T, int NT, typename I>
__global__ void __launch_bounds__(kRedThreads) pauli_group_kernel(const cplx<T>* __restrict__ sv, int n, int64_t sv_stride,
                                                                  const __grid_constant__ PauliGroup g, int nslots,
                                                                  double* __restrict__ partials) {
    const int64_t b = blockIdx.y;
    const cplx<T>* s = sv + b * sv_stride;
    const int nblk = gridDim.x;
    Acc<T, NT> acc;
    const I stride = I(nblk) * blockDim.x;
    I zm[NT];
#pragma unroll
    for (int j = 0; j < NT; ++j) zm[j] = I(g.zmask[j]);
    // grid-stride loops unrolled so that each thread has several independent loads in flight
    if (g.xmask == 0) {
        constexpr int U = 4;
        const I len = I(1) << n;
        for (I x0 = I(blockIdx.x) * blockDim.x + threadIdx.x; x0 < len; x0 += U * stride) {
            cplx<T> a[U];
#pragma unroll
            for (int u = 0; u < U; ++u) a[u] = x0 + u * stride < len ? s[x0 + u * stride] : mk<T>(T(0), T(0));
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const I x = x0 + u * stride;
                if (x >= len) break;
                const T p = a[u].x * a[u].x + a[u].y * a[u].y;
#pragma unroll
                for (int j = 0; j < NT; ++j)
                    if (j < g.nterms) acc.add(j, (popc_any(I(x & zm[j])) & 1) ? -p : p);
                acc.step();
            }
        }
    } else {
        // visit each pair {x, x ^ xmask} once: x has a zero at the top bit of xmask
        constexpr int U = 2;
        const int top = 63 - __clzll(g.xmask);
        const I xm = I(g.xmask);
        const I half = I(1) << (n - 1);
        for (I i0 = I(blockIdx.x) * blockDim.x + threadIdx.x; i0 < half; i0 += U * stride) {
            cplx<T> a[U], c[U];
            I xs[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const I i = i0 + u * stride;
                xs[u] = ((i >> top) << (top + 1)) | (i & ((I(1) << top) - 1));
                a[u] = c[u] = mk<T>(T(0), T(0));
                if (i < half) {
                    a[u] = s[xs[u]];
                    c[u] = s[xs[u] ^ xm];
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (i0 + u * stride >= half) break;
                const I x = xs[u], y = x ^ xm;
                // v = conj(psi[y]) psi[x] contributes at x; conj(v) contributes at y
                const T vr = c[u].x * a[u].x + c[u].y * a[u].y;
                const T vi = c[u].x * a[u].y - c[u].y * a[u].x;
#pragma unroll
                for (int j = 0; j < NT; ++j)
                    if (j < g.nterms) {
                        const T tx = re_iny<T>(vr, vi, g.ny[j]);
                        const T ty = re_iny<T>(vr, -vi, g.ny[j]);
                        acc.add(j, ((popc_any(I(x & zm[j])) & 1) ? -tx : tx) + ((popc_any(I(y & zm[j])) & 1) ? -ty : ty));
                    }
                acc.step();
            }
        }
    }
    acc.flush();
#pragma unroll
    for (int j = 0; j < NT; ++j) acc.d[j] *= g.coeff[j < g.nterms ? j : 0];
    double* dst = partials + (int64_t(b) * nslots + g.slot0) * nblk + blockIdx.x;
    block_reduce_store<NT>(acc.d, dst, nblk, g.nterms);
}

// out[b * nslots + t] = coeff[t] * sum_blk partials[(b * nslots + t) * nblk + blk]
__global__ void finish_kernel(const double* __restrict__ partials, int nblk, int nslots, int64_t batch,
                              const double* __restrict__ coeff, double* __restrict__ out) {
    const int64_t item = int64_t(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (item >= batch * nslots) return;
    const double* p = partials + item * nblk;
    double s = 0;
    for (int i = lane; i < nblk; i += 32) s += p[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[item] = s * (coeff ? coeff[item % nslots] : 1.0);
}

// Sum of |v|^2 (slot 0) -- normalize_state.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) norm2_kernel(const cplx<T>* __restrict__ sv, int n, int64_t sv_stride,
                                                            double* __restrict__ partials) {
    const cplx<T>* s = sv + int64_t(blockIdx.y) * sv_stride;
    const uint64_t len = uint64_t(1) << n, stride = uint64_t(gridDim.x) * blockDim.x;
    Acc<T, 1> acc;
    constexpr int U = 4;  // independent loads in flight per thread
    for (uint64_t x0 = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; x0 < len; x0 += U * stride) {
        cplx<T> a[U];
#pragma unroll
        for (int u = 0; u < U; ++u) a[u] = x0 + u * stride < len ? s[x0 + u * stride] : mk<T>(T(0), T(0));
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (x0 + u * stride >= len) break;
            acc.add(0, a[u].x * a[u].x + a[u].y * a[u].y);
            acc.step();
        }
    }
    acc.flush();
    block_reduce_store<1>(acc.d, partials + int64_t(blockIdx.y) * gridDim.x + blockIdx.x, gridDim.x);
}

// <a|b> = sum conj(a) b (slots 0, 1 = real, imaginary).
template <typename T>
__global__ void __launch_bounds__(kRedThreads) inner_kernel(const cplx<T>* __restrict__ a, const cplx<T>* __restrict__ bv,
                                                            int n, int64_t stride_ab, double* __restrict__ partials) {
    const int64_t b = blockIdx.y;
    const cplx<T>* x = a + b * stride_ab;
    const cplx<T>* y = bv + b * stride_ab;
    const uint64_t len = uint64_t(1) << n, stride = uint64_t(gridDim.x) * blockDim.x;
    Acc<T, 2> acc;
    constexpr int U = 2;  // independent loads in flight per thread
    for (uint64_t i0 = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i0 < len; i0 += U * stride) {
        cplx<T> us[U], vs[U];
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const uint64_t i = i0 + k * stride;
            us[k] = i < len ? x[i] : mk<T>(T(0), T(0));
            vs[k] = i < len ? y[i] : mk<T>(T(0), T(0));
        }
#pragma unroll
        for (int k = 0; k < U; ++k) {
            if (i0 + k * stride >= len) break;
            const cplx<T> u = us[k], v = vs[k];
            acc.add(0, u.x * v.x + u.y * v.y);
            acc.add(1, u.x * v.y - u.y * v.x);
            acc.step();
        }
    }
    acc.flush();
    block_reduce_store<2>(acc.d, partials + (b * 2) * gridDim.x + blockIdx.x, gridDim.x);
}

// Partial overlap on k <= 2 sites: slots 2*(r*D+c) (+1) = re/im of sum a[r,rest] conj(b[c,rest]).
struct OverlapArgs {
    int n, k;
    int sorted[2];
    uint32_t off[4];
};

template <typename T, int K>
__global__ void __launch_bounds__(kRedThreads) overlap_kernel(const cplx<T>* __restrict__ a, const cplx<T>* __restrict__ bv,
                                                              int64_t stride_ab, const __grid_constant__ OverlapArgs o,
                                                              double* __restrict__ partials) {
    constexpr int D = 1 << K;
    const int64_t b = blockIdx.y;
    const cplx<T>* x = a + b * stride_ab;
    const cplx<T>* y = bv + b * stride_ab;
    const uint64_t groups = uint64_t(1) << (o.n - K), stride = uint64_t(gridDim.x) * blockDim.x;
    Acc<T, 2 * D * D> acc;
    for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < groups; g += stride) {
        uint64_t base = g;
#pragma unroll
        for (int j = 0; j < K; ++j) base = ((base >> o.sorted[j]) << (o.sorted[j] + 1)) | (base & ((uint64_t(1) << o.sorted[j]) - 1));
        cplx<T> u[D], v[D];
#pragma unroll
        for (int r = 0; r < D; ++r) {
            u[r] = x[base + o.off[r]];
            v[r] = y[base + o.off[r]];
        }
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int c = 0; c < D; ++c) {
                // u[r] * conj(v[c])
                acc.add(2 * (r * D + c), u[r].x * v[c].x + u[r].y * v[c].y);
                acc.add(2 * (r * D + c) + 1, u[r].y * v[c].x - u[r].x * v[c].y);
            }
        acc.step();
    }
    acc.flush();
    block_reduce_store<2 * D * D>(acc.d, partials + (b * 2 * D * D) * gridDim.x + blockIdx.x, gridDim.x);
}

// Partial overlap on any k <= kOvlMaxK sites: a warp per (row r, column c,
// chunk of the other bits) sums a[r, rest] conj(b[c, rest]) with lane-strided
// reads (Acc rule, fixed xor tree); the chunks of a pair are added in order by
// finish(). partials[((bt * pairs + pair) * 2 + re/im) * chunks + chunk].
constexpr int kOvlMaxK = 10;

struct OvlArgs {
    int n, k;
    int pos[kOvlMaxK];     // flat bit of matrix bit (k-1-j), j = 0 .. k-1
    int sorted[kOvlMaxK];  // the same bits ascending
    uint64_t chunks, chunk;  // chunks per pair, rest values per chunk
};

__host__ __device__ inline uint64_t ovl_chunks(int n, int k) {
    // about 2^22 / 4^k warps (at least one chunk), each chunk at least 1024 values
    const uint64_t rest = uint64_t(1) << (n - k);
    uint64_t c = rest / 1024;
    const uint64_t cap = (uint64_t(1) << 22) >> (2 * k);
    if (c > cap) c = cap;
    return c < 1 ? 1 : c;
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) overlap_pair_kernel(const cplx<T>* __restrict__ a,
                                                                   const cplx<T>* __restrict__ bv, int64_t stride_ab,
                                                                   const __grid_constant__ OvlArgs o,
                                                                   double* __restrict__ partials) {
    const uint64_t w = (uint64_t(blockIdx.x) * kRedThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint64_t pairs = uint64_t(1) << (2 * o.k);
    if (w >= pairs * o.chunks) return;  // whole warps leave together
    const int64_t bt = blockIdx.y;
    const cplx<T>* x = a + bt * stride_ab;
    const cplx<T>* y = bv + bt * stride_ab;
    const uint64_t pair = w / o.chunks, ch = w - pair * o.chunks;
    const int r = int(pair >> o.k), c = int(pair & ((uint64_t(1) << o.k) - 1));
    const uint64_t offr = matrix_offset(r, o.pos, o.k), offc = matrix_offset(c, o.pos, o.k);
    Acc<T, 2> acc;
    for (uint64_t t = ch * o.chunk + lane; t < (ch + 1) * o.chunk; t += 32) {
        const uint64_t base = insert_zeros(t, o.sorted, o.k);
        const cplx<T> u = x[base | offr], v = y[base | offc];
        acc.add(0, u.x * v.x + u.y * v.y);  // u conj(v)
        acc.add(1, u.y * v.x - u.x * v.y);
        acc.step();
    }
    acc.flush();
    double re = acc.d[0], im = acc.d[1];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, off);
        im += __shfl_xor_sync(0xffffffffu, im, off);
    }
    if (lane == 0) {
        double* p = partials + ((uint64_t(bt) * pairs + pair) * 2) * o.chunks + ch;
        p[0] = re;
        p[o.chunks] = im;
    }
}

// DM: Tr(rho P) for one Pauli group: sum_x rho[x, x ^ xmask] i^ny (-1)^{pop(x & zmask)}.
template <typename T, int NT>
__global__ void __launch_bounds__(kRedThreads) dm_pauli_kernel(const cplx<T>* __restrict__ rho, int n, int64_t stride,
                                                               const __grid_constant__ PauliGroup g, int nslots,
                                                               double* __restrict__ partials) {
    const int64_t b = blockIdx.y;
    const cplx<T>* r = rho + b * stride;
    const uint64_t dim = uint64_t(1) << n, step = uint64_t(gridDim.x) * blockDim.x;
    Acc<T, NT> acc;
    for (uint64_t x = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; x < dim; x += step) {
        const cplx<T> v = r[(x << n) | (x ^ g.xmask)];
#pragma unroll
        for (int j = 0; j < NT; ++j)
            if (j < g.nterms) {
                const T t = re_iny<T>(v.x, v.y, g.ny[j]);
                acc.add(j, (__popcll(x & g.zmask[j]) & 1) ? -t : t);
            }
        acc.step();
    }
    acc.flush();
#pragma unroll
    for (int j = 0; j < NT; ++j) acc.d[j] *= g.coeff[j < g.nterms ? j : 0];
    block_reduce_store<NT>(acc.d, partials + (int64_t(b) * nslots + g.slot0) * gridDim.x + blockIdx.x, gridDim.x,
                           g.nterms);
}

// DM: Re Tr((x)_q O_q rho) = Re sum_{x,y} prod_q O_q[x_q, y_q] rho[y, x].
struct ProductOps {
    int n;
    double2 o[QGB_MAX_QUBITS][4];  // o[q][2*a + b] = O_q[a][b]
};

template <typename T>
__global__ void __launch_bounds__(kRedThreads) dm_product_kernel(const cplx<T>* __restrict__ rho, int64_t stride,
                                                                 const __grid_constant__ ProductOps p,
                                                                 double* __restrict__ partials) {
    const int n = p.n;
    const cplx<T>* r = rho + int64_t(blockIdx.y) * stride;
    const uint64_t len = uint64_t(1) << (2 * n), step = uint64_t(gridDim.x) * blockDim.x;
    const uint64_t lo = (uint64_t(1) << n) - 1;
    Acc<T, 1> acc;
    for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < len; v += step) {
        const uint64_t y = v >> n, x = v & lo;  // entry rho[y, x]
        T wr = T(1), wi = T(0);
        for (int q = 0; q < n; ++q) {
            const int xa = int((x >> (n - 1 - q)) & 1), yb = int((y >> (n - 1 - q)) & 1);
            const double2 c = p.o[q][2 * xa + yb];
            const T tr = wr * T(c.x) - wi * T(c.y);
            wi = wr * T(c.y) + wi * T(c.x);
            wr = tr;
        }
        const cplx<T> e = r[v];
        acc.add(0, wr * e.x - wi * e.y);
        acc.step();
    }
    acc.flush();
    block_reduce_store<1>(acc.d, partials + int64_t(blockIdx.y) * gridDim.x + blockIdx.x, gridDim.x);
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) dm_trace_kernel(const cplx<T>* __restrict__ rho, int n, int64_t stride,
                                                               double* __restrict__ partials) {
    const cplx<T>* r = rho + int64_t(blockIdx.y) * stride;
    const uint64_t dim = uint64_t(1) << n, step = uint64_t(gridDim.x) * blockDim.x;
    Acc<T, 1> acc;
    for (uint64_t x = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; x < dim; x += step) {
        acc.add(0, r[(x << n) | x].x);
        acc.step();
    }
    acc.flush();
    block_reduce_store<1>(acc.d, partials + int64_t(blockIdx.y) * gridDim.x + blockIdx.x, gridDim.x);
}

// Trace chain of a complex64 density matrix run on the tensor cores: the tensor
// cores accumulate with round-toward-zero, so every pass shrinks vec(rho) by
// ~1e-7 of its size, and a channel (unlike a unitary) keeps no vector norm that
// could be restored. A channel sequence keeps the trace instead: one CTA sums
// the 2^n diagonal entries (index x (2^n + 1)) in float64 in a fixed order and
// writes chain[0] = that trace (start) or chain[1] = chain[0] / trace, the
// factor the next plain tensor-core pass folds into its matrix; chain[2] keeps
// the measured trace.
template <typename T>
__global__ void __launch_bounds__(1024) trace_factor_kernel(const cplx<T>* __restrict__ rho, int n,
                                                            double* __restrict__ chain, int start) {
    __shared__ double red[32];
    const uint64_t dim = uint64_t(1) << n;
    double s = 0.0;
#pragma unroll 4
    for (uint64_t x = threadIdx.x; x < dim; x += blockDim.x) s += double(rho[(x << n) | x].x);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) t += red[w];
        if (start) {
            chain[0] = t;
            chain[1] = 1.0;
        } else {
            const double ref = chain[0];
            chain[1] = (ref > 0.0 && t > 0.0) ? ref / t : 1.0;
        }
        chain[2] = t;
    }
}

// Adjoint reverse step for one gate U on K <= 2 sites, one pass over two vectors:
//   phi <- U^dagger phi,  lam <- U^dagger lam, and, by GradMode,
//   kGradNone:     nothing else;
//   kGradMatrix:   grad[r][c] += lam[r] * conj(phi_new[c]) (slots 2*(r*D+c) (+1) =
//                  re/im; the host scales by 2, torch's convention);
//   kGradRotation: for U = exp(-i theta P) (P^2 = I): one slot,
//                  Im sum_r conj(lam[r]) (P phi)[r] with phi, lam taken at the
//                  gate's output (before the uncompute). Since U commutes with P,
//                  Re sum_rc conj(G[r,c]) dU/dtheta[r,c] = 2 Im <lam|P|phi> for
//                  G = 2 sum lam[r] conj(phi_new[c]): the angle's gradient
//                  without the 2 D^2 matrix-gradient slots.
enum GradMode { kGradNone = 0, kGradMatrix = 1, kGradRotation = 2 };

struct AdjointArgs {
    int n;
    int sorted[2];
    uint32_t off[4];
    int64_t sv_stride;  // batch: state b at phi + b * sv_stride (and lam)
    int64_t op_stride;  // batch: its gate matrix at U + b * op_stride
    int gcol[4];        // kGradRotation: P[r][gcol[r]] = gval[r], the only nonzero of row r
    double2 gval[4];
};

template <int K, int MODE>
__host__ __device__ constexpr int adjoint_slots() {
    return MODE == kGradMatrix ? (2 << (2 * K)) : 1;
}

template <typename T, int K, int MODE>
__global__ void __launch_bounds__(kRedThreads) adjoint_kernel(cplx<T>* __restrict__ phi, cplx<T>* __restrict__ lam,
                                                              const cplx<T>* __restrict__ U,
                                                              const __grid_constant__ AdjointArgs a,
                                                              double* __restrict__ partials) {
    constexpr int D = 1 << K;
    constexpr int NS = adjoint_slots<K, MODE>();
    using C = cplx<T>;
    const int64_t bidx = blockIdx.y;  // state of the batch
    phi += bidx * a.sv_stride;
    lam += bidx * a.sv_stride;
    U += bidx * a.op_stride;
    C ud[D * D];  // U^dagger
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const C u = U[c * D + r];
            ud[r * D + c] = mk<T>(u.x, -u.y);
        }
    const uint64_t groups = uint64_t(1) << (a.n - K), stride = uint64_t(gridDim.x) * blockDim.x;
    C gv[D];  // kGradRotation: the nonzero of each row of P, in the state's precision
    int gc[D];
#pragma unroll
    for (int r = 0; r < D; ++r) {
        gv[r] = mk<T>(T(a.gval[r].x), T(a.gval[r].y));
        gc[r] = a.gcol[r];
    }
    Acc<T, NS> acc;
    for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < groups; g += stride) {
        uint64_t base = g;
#pragma unroll
        for (int j = 0; j < K; ++j) base = ((base >> a.sorted[j]) << (a.sorted[j] + 1)) | (base & ((uint64_t(1) << a.sorted[j]) - 1));
        C p[D], l[D], pn[D], ln[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            p[c] = phi[base + a.off[c]];
            l[c] = lam[base + a.off[c]];
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            C x = mk<T>(0, 0), y = mk<T>(0, 0);
#pragma unroll
            for (int c = 0; c < D; ++c) {
                cfma(x, ud[r * D + c], p[c]);
                cfma(y, ud[r * D + c], l[c]);
            }
            pn[r] = x;
            ln[r] = y;
        }
        if constexpr (MODE == kGradMatrix) {
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    acc.add(2 * (r * D + c), l[r].x * pn[c].x + l[r].y * pn[c].y);
                    acc.add(2 * (r * D + c) + 1, l[r].y * pn[c].x - l[r].x * pn[c].y);
                }
            acc.step();
        } else if constexpr (MODE == kGradRotation) {
            T s = T(0);
#pragma unroll
            for (int r = 0; r < D; ++r) {
                C pc = p[0];  // p[gc[r]] by selects (no dynamic register indexing)
#pragma unroll
                for (int c = 1; c < D; ++c)
                    if (gc[r] == c) pc = p[c];
                C w = mk<T>(0, 0);
                cfma(w, gv[r], pc);
                s += l[r].x * w.y - l[r].y * w.x;  // Im(conj(l) w)
            }
            acc.add(0, s);
            acc.step();
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            phi[base + a.off[r]] = pn[r];
            lam[base + a.off[r]] = ln[r];
        }
    }
    // partials[(b * slots + slot) * nblk + blk], the layout finish() sums
    if constexpr (MODE != kGradNone) {
        acc.flush();
        block_reduce_store<NS>(acc.d, partials + bidx * NS * gridDim.x + blockIdx.x, gridDim.x);
    }
}

// out = sum_t coeff[t] P_t sv
struct PauliApplyArgs {
    int n, nterms;
    uint64_t xmask[128], zmask[128];
    int ny[128];
    double coeff[128];
};

template <typename T>
__global__ void __launch_bounds__(256) pauli_apply_kernel(const cplx<T>* __restrict__ sv, cplx<T>* __restrict__ out,
                                                          int64_t stride, const __grid_constant__ PauliApplyArgs a) {
    const int64_t b = blockIdx.y;
    const cplx<T>* s = sv + b * stride;
    cplx<T>* o = out + b * stride;
    const uint64_t len = uint64_t(1) << a.n, step = uint64_t(gridDim.x) * blockDim.x;
    // computed in the state's own precision (the sum is rounded to it anyway)
    for (uint64_t y = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; y < len; y += step) {
        T ar = T(0), ai = T(0);
        for (int t = 0; t < a.nterms; ++t) {
            const uint64_t x = y ^ a.xmask[t];
            const cplx<T> v = s[x];
            // P|x> = i^ny (-1)^{pop(x & z)} |x ^ xmask> ; contribution to out[y]
            T cr = v.x, ci = v.y;
            switch (a.ny[t] & 3) {
                case 1: { T t2 = cr; cr = -ci; ci = t2; } break;
                case 2: cr = -cr; ci = -ci; break;
                case 3: { T t2 = cr; cr = ci; ci = -t2; } break;
                default: break;
            }
            const T f = T((__popcll(x & a.zmask[t]) & 1) ? -a.coeff[t] : a.coeff[t]);
            ar += f * cr;
            ai += f * ci;
        }
        o[y] = mk<T>(ar, ai);
    }
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

namespace {

struct ParsedPauli {
    uint64_t x, z;
    int ny;
};

int parse_paulis(const char* paulis, int n, int nterms, std::vector<ParsedPauli>& out) {
    if (!paulis) return set_error(QGB_EINVAL, "null Pauli strings");
    if (n > 64) return set_error(QGB_EINVAL, "Pauli strings limited to 64 sites");
    out.resize(nterms);
    for (int t = 0; t < nterms; ++t) {
        ParsedPauli p{0, 0, 0};
        for (int q = 0; q < n; ++q) {
            const uint64_t bit = 1ull << (n - 1 - q);
            switch (paulis[size_t(t) * n + q]) {
                case 'i': case 'I': break;
                case 'x': case 'X': p.x |= bit; break;
                case 'y': case 'Y': p.x |= bit; p.z |= bit; p.ny++; break;
                case 'z': case 'Z': p.z |= bit; break;
                default: return set_error(QGB_EINVAL, "invalid Pauli character in term %d", t);
            }
        }
        out[t] = p;
    }
    return QGB_OK;
}

size_t red_scratch(int nbits, int nslots, int64_t batch) {
    return sizeof(double) * size_t(red_blocks(nbits)) * size_t(nslots) * size_t(batch);
}

int check_common(const void* p, int dtype, int nbits, int64_t batch, int64_t stride) {
    if (!p) return set_error(QGB_EINVAL, "null state");
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    if (nbits < 1 || nbits > 2 * QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid", nbits);
    if (batch < 1 || batch > 65535) return set_error(QGB_EINVAL, "batch out of range");
    if (batch > 1 && stride < (int64_t(1) << nbits)) return set_error(QGB_EINVAL, "stride smaller than the state");
    return QGB_OK;
}

int finish(const double* partials, int nblk, int nslots, int64_t batch, const double* coeff, double* out, cudaStream_t st) {
    const int64_t items = batch * nslots;
    const unsigned blocks = unsigned((items + 7) / 8);
    finish_kernel<<<blocks, 256, 0, st>>>(partials, nblk, nslots, batch, coeff, out);
    return check_launch("reduction finish");
}

template <typename T, int NT>
void launch_group(const void* sv, int n, int64_t stride, const PauliGroup& g, int nslots, double* partials,
                  int64_t batch, bool dm, cudaStream_t st) {
    const int nbits = dm ? 2 * n : n;
    dim3 grid(red_blocks(nbits), unsigned(batch));
    if (dm)
        dm_pauli_kernel<T, NT><<<grid, kRedThreads, 0, st>>>((const cplx<T>*)sv, n, stride, g, nslots, partials);
    else if (n <= 31)
        pauli_group_kernel<T, NT, uint32_t><<<grid, kRedThreads, 0, st>>>((const cplx<T>*)sv, n, stride, g, nslots,
                                                                          partials);
    else
        pauli_group_kernel<T, NT, uint64_t><<<grid, kRedThreads, 0, st>>>((const cplx<T>*)sv, n, stride, g, nslots,
                                                                          partials);
}

template <typename T>
void launch_group_nt(const void* sv, int n, int64_t stride, const PauliGroup& g, int nslots, double* partials,
                     int64_t batch, bool dm, cudaStream_t st) {
    if (g.nterms <= 1) launch_group<T, 1>(sv, n, stride, g, nslots, partials, batch, dm, st);
    else if (g.nterms <= 4) launch_group<T, 4>(sv, n, stride, g, nslots, partials, batch, dm, st);
    else if (g.nterms <= 8) launch_group<T, 8>(sv, n, stride, g, nslots, partials, batch, dm, st);
    else launch_group<T, 32>(sv, n, stride, g, nslots, partials, batch, dm, st);
}

int pauli_expect_impl(const void* sv, int dtype, int n, const char* paulis, const double* coeff, int nterms,
                      int64_t batch, int64_t stride, double* out, void* scratch, size_t scratch_bytes, bool dm,
                      cudaStream_t st) {
    const int nbits = dm ? 2 * n : n;
    int rc = check_common(sv, dtype, nbits, batch, stride);
    if (rc) return rc;
    if (!out) return set_error(QGB_EINVAL, "null output");
    if (nterms < 1) return set_error(QGB_EINVAL, "no terms");
    if (!scratch || scratch_bytes < red_scratch(nbits, nterms, batch))
        return set_error(QGB_ESCRATCH, "scratch of %zu bytes needed", red_scratch(nbits, nterms, batch));
    std::vector<ParsedPauli> ps;
    if ((rc = parse_paulis(paulis, n, nterms, ps))) return rc;
    // Output slot t belongs to term t; terms are grouped by X mask (<= 32 per launch)
    // and each group's slots must be contiguous: process terms in an order where
    // each launch covers a contiguous run of slots with a common X mask.
    double* partials = (double*)scratch;
    int t = 0;
    while (t < nterms) {
        PauliGroup g{};
        g.xmask = ps[t].x;
        g.slot0 = t;
        g.nterms = 0;
        while (t < nterms && ps[t].x == g.xmask && g.nterms < 32) {
            g.zmask[g.nterms] = ps[t].z;
            g.ny[g.nterms] = ps[t].ny;
            g.coeff[g.nterms] = coeff ? coeff[t] : 1.0;
            ++g.nterms;
            ++t;
        }
        if (dtype == QGB_C64) launch_group_nt<float>(sv, n, stride, g, nterms, partials, batch, dm, st);
        else launch_group_nt<double>(sv, n, stride, g, nterms, partials, batch, dm, st);
        if ((rc = check_launch("pauli expectation"))) return rc;
    }
    return finish(partials, red_blocks(nbits), nterms, batch, nullptr, out, st);
}

}  // namespace

extern "C" size_t qgb_reduce_scratch_bytes(int n, int nterms, int64_t batch) {
    if (n < 1 || n > 2 * QGB_MAX_QUBITS || nterms < 1 || batch < 1) return 0;
    // the largest reduction over 2^n entries (n already doubled by DM callers)
    int slots = nterms < 32 ? 32 : nterms;  // partial overlap on 2 sites needs 32 slots
    return red_scratch(n, slots, batch);
}

extern "C" int qgb_norm2(const void* sv, int dtype, int n, int64_t batch, int64_t sv_stride, double* out, void* scratch,
                         size_t scratch_bytes, void* stream) {
    int rc = check_common(sv, dtype, n, batch, sv_stride);
    if (rc) return rc;
    if (!out) return set_error(QGB_EINVAL, "null output");
    if (!scratch || scratch_bytes < red_scratch(n, 1, batch)) return set_error(QGB_ESCRATCH, "scratch too small");
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid(red_blocks(n), unsigned(batch));
    if (dtype == QGB_C64) norm2_kernel<float><<<grid, kRedThreads, 0, st>>>((const float2*)sv, n, sv_stride, (double*)scratch);
    else norm2_kernel<double><<<grid, kRedThreads, 0, st>>>((const double2*)sv, n, sv_stride, (double*)scratch);
    if ((rc = check_launch("norm2"))) return rc;
    return finish((const double*)scratch, red_blocks(n), 1, batch, nullptr, out, st);
}

extern "C" int qgb_inner_product(const void* a, const void* b, int dtype, int n, int64_t batch, int64_t stride,
                                 double* out, void* scratch, size_t scratch_bytes, void* stream) {
    int rc = check_common(a, dtype, n, batch, stride);
    if (rc) return rc;
    if (!b || !out) return set_error(QGB_EINVAL, "null pointer");
    if (!scratch || scratch_bytes < red_scratch(n, 2, batch)) return set_error(QGB_ESCRATCH, "scratch too small");
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid(red_blocks(n), unsigned(batch));
    if (dtype == QGB_C64)
        inner_kernel<float><<<grid, kRedThreads, 0, st>>>((const float2*)a, (const float2*)b, n, stride, (double*)scratch);
    else
        inner_kernel<double><<<grid, kRedThreads, 0, st>>>((const double2*)a, (const double2*)b, n, stride, (double*)scratch);
    if ((rc = check_launch("inner product"))) return rc;
    return finish((const double*)scratch, red_blocks(n), 2, batch, nullptr, out, st);
}

extern "C" int qgb_pauli_expectation(const void* sv, int dtype, int n, const char* paulis, const double* coeff,
                                     int nterms, int64_t batch, int64_t sv_stride, double* out, void* scratch,
                                     size_t scratch_bytes, void* stream) {
    return pauli_expect_impl(sv, dtype, n, paulis, coeff, nterms, batch, sv_stride, out, scratch, scratch_bytes, false,
                             (cudaStream_t)stream);
}

extern "C" int qgb_dm_pauli_expectation(const void* rho, int dtype, int n, const char* paulis, const double* coeff,
                                        int nterms, int64_t batch, int64_t rho_stride, double* out, void* scratch,
                                        size_t scratch_bytes, void* stream) {
    return pauli_expect_impl(rho, dtype, n, paulis, coeff, nterms, batch, rho_stride, out, scratch, scratch_bytes, true,
                             (cudaStream_t)stream);
}

extern "C" size_t qgb_partial_overlap_scratch_bytes(int n, int k, int64_t batch) {
    if (n < 1 || n > 2 * QGB_MAX_QUBITS || k < 1 || k > n || k > kOvlMaxK || batch < 1) return 0;
    if (k <= 2) return red_scratch(n, 2 << (2 * k), batch);
    return sizeof(double) * size_t(batch) * (size_t(2) << (2 * k)) * size_t(ovl_chunks(n, k));
}

namespace {

// k > 2: the warp-per-pair kernel.
int partial_overlap_wide(const void* a, const void* b, int dtype, int n, const int* indices, int k, int64_t batch,
                         int64_t sv_stride, double* out, void* scratch, size_t scratch_bytes, cudaStream_t st) {
    OvlArgs o{};
    o.n = n;
    o.k = k;
    uint64_t seen = 0;
    for (int j = 0; j < k; ++j) {
        if (indices[j] < 0 || indices[j] >= n) return set_error(QGB_EINVAL, "site out of range");
        const int p = n - 1 - indices[j];
        if ((seen >> p) & 1ull) return set_error(QGB_EINVAL, "repeated site");
        seen |= 1ull << p;
        o.pos[j] = o.sorted[j] = p;
    }
    for (int i = 1; i < k; ++i)
        for (int j = i; j > 0 && o.sorted[j - 1] > o.sorted[j]; --j) {
            const int t = o.sorted[j];
            o.sorted[j] = o.sorted[j - 1];
            o.sorted[j - 1] = t;
        }
    o.chunks = ovl_chunks(n, k);
    o.chunk = (uint64_t(1) << (n - k)) / o.chunks;
    const uint64_t pairs = uint64_t(1) << (2 * k);
    const size_t need = sizeof(double) * size_t(batch) * size_t(2 * pairs) * size_t(o.chunks);
    if (!scratch || scratch_bytes < need)
        return set_error(QGB_ESCRATCH, "scratch of %zu bytes needed (qgb_partial_overlap_scratch_bytes)", need);
    const uint64_t blocks = (pairs * o.chunks * 32 + kRedThreads - 1) / kRedThreads;
    if (blocks > 0x7fffffffull) return set_error(QGB_EINVAL, "partial overlap too large");
    const dim3 grid(static_cast<unsigned>(blocks), static_cast<unsigned>(batch));
    if (dtype == QGB_C64)
        overlap_pair_kernel<float><<<grid, kRedThreads, 0, st>>>((const float2*)a, (const float2*)b, sv_stride, o,
                                                                 (double*)scratch);
    else
        overlap_pair_kernel<double><<<grid, kRedThreads, 0, st>>>((const double2*)a, (const double2*)b, sv_stride, o,
                                                                  (double*)scratch);
    int rc = check_launch("partial overlap (wide)");
    if (rc) return rc;
    // out[bt * 2 pairs + 2 pair + re/im] = sum over chunks: the same layout as the k <= 2 path
    return finish((const double*)scratch, int(o.chunks), int(2 * pairs), batch, nullptr, out, st);
}

}  // namespace

extern "C" int qgb_partial_overlap(const void* a, const void* b, int dtype, int n, const int* indices, int k,
                                   int64_t batch, int64_t sv_stride, double* out, void* scratch, size_t scratch_bytes,
                                   void* stream) {
    int rc = check_common(a, dtype, n, batch, sv_stride);
    if (rc) return rc;
    if (!b || !out || !indices) return set_error(QGB_EINVAL, "null pointer");
    if (k < 1 || k > n || k > kOvlMaxK)
        return set_error(QGB_EINVAL, "partial overlap supports 1 to %d sites (k=%d)", kOvlMaxK, k);
    if (k > 2)
        return partial_overlap_wide(a, b, dtype, n, indices, k, batch, sv_stride, out, scratch, scratch_bytes,
                                    (cudaStream_t)stream);
    const int slots = 2 << (2 * k);
    if (!scratch || scratch_bytes < red_scratch(n, slots, batch)) return set_error(QGB_ESCRATCH, "scratch too small");
    OverlapArgs o{};
    o.n = n;
    o.k = k;
    int pos[2];
    for (int j = 0; j < k; ++j) {
        if (indices[j] < 0 || indices[j] >= n) return set_error(QGB_EINVAL, "site out of range");
        pos[j] = n - 1 - indices[j];
        o.sorted[j] = pos[j];
    }
    if (k == 2) {
        if (pos[0] == pos[1]) return set_error(QGB_EINVAL, "repeated site");
        if (o.sorted[0] > o.sorted[1]) { int t = o.sorted[0]; o.sorted[0] = o.sorted[1]; o.sorted[1] = t; }
    }
    for (int r = 0; r < (1 << k); ++r) o.off[r] = uint32_t(matrix_offset(r, pos, k));
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid(red_blocks(n), unsigned(batch));
    if (dtype == QGB_C64) {
        if (k == 1) overlap_kernel<float, 1><<<grid, kRedThreads, 0, st>>>((const float2*)a, (const float2*)b, sv_stride, o, (double*)scratch);
        else overlap_kernel<float, 2><<<grid, kRedThreads, 0, st>>>((const float2*)a, (const float2*)b, sv_stride, o, (double*)scratch);
    } else {
        if (k == 1) overlap_kernel<double, 1><<<grid, kRedThreads, 0, st>>>((const double2*)a, (const double2*)b, sv_stride, o, (double*)scratch);
        else overlap_kernel<double, 2><<<grid, kRedThreads, 0, st>>>((const double2*)a, (const double2*)b, sv_stride, o, (double*)scratch);
    }
    if ((rc = check_launch("partial overlap"))) return rc;
    return finish((const double*)scratch, red_blocks(n), slots, batch, nullptr, out, st);
}

extern "C" int qgb_dm_product_expectation(const void* rho, int dtype, int n, const double* ops, int64_t batch,
                                          int64_t rho_stride, double* out, void* scratch, size_t scratch_bytes,
                                          void* stream) {
    int rc = check_common(rho, dtype, 2 * n, batch, rho_stride);
    if (rc) return rc;
    if (!ops || !out) return set_error(QGB_EINVAL, "null pointer");
    if (n > QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n too large");
    if (!scratch || scratch_bytes < red_scratch(2 * n, 1, batch)) return set_error(QGB_ESCRATCH, "scratch too small");
    ProductOps p{};
    p.n = n;
    for (int q = 0; q < n; ++q)
        for (int e = 0; e < 4; ++e) p.o[q][e] = make_double2(ops[(q * 4 + e) * 2], ops[(q * 4 + e) * 2 + 1]);
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid(red_blocks(2 * n), unsigned(batch));
    if (dtype == QGB_C64) dm_product_kernel<float><<<grid, kRedThreads, 0, st>>>((const float2*)rho, rho_stride, p, (double*)scratch);
    else dm_product_kernel<double><<<grid, kRedThreads, 0, st>>>((const double2*)rho, rho_stride, p, (double*)scratch);
    if ((rc = check_launch("dm product expectation"))) return rc;
    return finish((const double*)scratch, red_blocks(2 * n), 1, batch, nullptr, out, st);
}

extern "C" int qgb_dm_trace(const void* rho, int dtype, int n, int64_t batch, int64_t rho_stride, double* out,
                            void* scratch, size_t scratch_bytes, void* stream) {
    int rc = check_common(rho, dtype, 2 * n, batch, rho_stride);
    if (rc) return rc;
    if (!out) return set_error(QGB_EINVAL, "null output");
    if (!scratch || scratch_bytes < red_scratch(2 * n, 1, batch)) return set_error(QGB_ESCRATCH, "scratch too small");
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid(red_blocks(2 * n), unsigned(batch));
    if (dtype == QGB_C64) dm_trace_kernel<float><<<grid, kRedThreads, 0, st>>>((const float2*)rho, n, rho_stride, (double*)scratch);
    else dm_trace_kernel<double><<<grid, kRedThreads, 0, st>>>((const double2*)rho, n, rho_stride, (double*)scratch);
    if ((rc = check_launch("dm trace"))) return rc;
    return finish((const double*)scratch, red_blocks(2 * n), 1, batch, nullptr, out, st);
}

extern "C" int qgb_dm_trace_factor(const void* rho, int dtype, int n, double* chain, int start, void* stream) {
    int rc = check_common(rho, dtype, 2 * n, 1, 0);
    if (rc) return rc;
    if (!chain || (reinterpret_cast<uintptr_t>(chain) % sizeof(double)))
        return set_error(QGB_EINVAL, "chain buffer missing or not 8-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == QGB_C64) trace_factor_kernel<float><<<1, 1024, 0, st>>>((const float2*)rho, n, chain, start);
    else trace_factor_kernel<double><<<1, 1024, 0, st>>>((const double2*)rho, n, chain, start);
    return check_launch("dm trace factor");
}

extern "C" int qgb_pauli_apply(const void* sv, void* out, int dtype, int n, const char* paulis, const double* coeff,
                               int nterms, int64_t batch, int64_t sv_stride, void* stream) {
    int rc = check_common(sv, dtype, n, batch, sv_stride);
    if (rc) return rc;
    if (!out || !coeff) return set_error(QGB_EINVAL, "null pointer");
    if (out == sv) return set_error(QGB_EINVAL, "output must not alias the input");
    if (nterms < 1 || nterms > 128) return set_error(QGB_EINVAL, "1..128 terms supported (got %d)", nterms);
    std::vector<ParsedPauli> ps;
    if ((rc = parse_paulis(paulis, n, nterms, ps))) return rc;
    PauliApplyArgs a{};
    a.n = n;
    a.nterms = nterms;
    for (int t = 0; t < nterms; ++t) {
        a.xmask[t] = ps[t].x;
        a.zmask[t] = ps[t].z;
        a.ny[t] = ps[t].ny;
        a.coeff[t] = coeff[t];
    }
    cudaStream_t st = (cudaStream_t)stream;
    const uint64_t len = uint64_t(1) << n;
    uint64_t bx = (len + 255) / 256;
    const uint64_t cap = uint64_t(sm_count()) * 8;
    if (bx > cap) bx = cap;
    dim3 grid((unsigned)bx, (unsigned)batch);
    if (dtype == QGB_C64) pauli_apply_kernel<float><<<grid, 256, 0, st>>>((const float2*)sv, (float2*)out, sv_stride, a);
    else pauli_apply_kernel<double><<<grid, 256, 0, st>>>((const double2*)sv, (double2*)out, sv_stride, a);
    return check_launch("pauli apply");
}

namespace {

template <int MODE>
void launch_adjoint(void* phi, void* lam, int dtype, int k, const void* op, const AdjointArgs& a, dim3 grid,
                    double* part, cudaStream_t st) {
    if (dtype == QGB_C64) {
        if (k == 1) adjoint_kernel<float, 1, MODE><<<grid, kRedThreads, 0, st>>>((float2*)phi, (float2*)lam, (const float2*)op, a, part);
        else adjoint_kernel<float, 2, MODE><<<grid, kRedThreads, 0, st>>>((float2*)phi, (float2*)lam, (const float2*)op, a, part);
    } else {
        if (k == 1) adjoint_kernel<double, 1, MODE><<<grid, kRedThreads, 0, st>>>((double2*)phi, (double2*)lam, (const double2*)op, a, part);
        else adjoint_kernel<double, 2, MODE><<<grid, kRedThreads, 0, st>>>((double2*)phi, (double2*)lam, (const double2*)op, a, part);
    }
}

// Shared checks and launch of the three adjoint-step forms.
int adjoint_impl(void* phi, void* lam, int dtype, int n, const int* indices, int k, const void* op, int64_t op_stride,
                 int64_t batch, int64_t sv_stride, const double* generator, double* grad_out, void* scratch,
                 size_t scratch_bytes, cudaStream_t st) {
    int rc = check_common(phi, dtype, n, batch, sv_stride);
    if (rc) return rc;
    if (!lam || !op || !indices) return set_error(QGB_EINVAL, "null pointer");
    if (lam == phi) return set_error(QGB_EINVAL, "the two vectors must be distinct");
    if (k < 1 || k > 2 || k > n) return set_error(QGB_EINVAL, "adjoint steps support gates on 1 or 2 sites (k=%d)", k);
    if (op_stride < 0) return set_error(QGB_EINVAL, "negative operator stride");
    const int64_t span = (batch - 1) * (sv_stride > 0 ? sv_stride : 0) + (int64_t(1) << n);
    const char* pb = static_cast<const char*>(phi);
    const char* lb = static_cast<const char*>(lam);
    const int64_t esz = dtype == QGB_C64 ? 8 : 16;
    if (pb < lb + span * esz && lb < pb + span * esz) return set_error(QGB_EINVAL, "the two batches overlap");
    const int mode = !grad_out ? kGradNone : (generator ? kGradRotation : kGradMatrix);
    const int slots = mode == kGradMatrix ? 2 << (2 * k) : 1;
    if (mode != kGradNone && (!scratch || scratch_bytes < red_scratch(n, slots, batch)))
        return set_error(QGB_ESCRATCH, "scratch too small");
    AdjointArgs a{};
    a.n = n;
    a.sv_stride = batch > 1 ? sv_stride : 0;
    a.op_stride = batch > 1 ? op_stride : 0;
    int pos[2];
    for (int j = 0; j < k; ++j) {
        if (indices[j] < 0 || indices[j] >= n) return set_error(QGB_EINVAL, "site out of range");
        pos[j] = n - 1 - indices[j];
        a.sorted[j] = pos[j];
    }
    if (k == 2) {
        if (pos[0] == pos[1]) return set_error(QGB_EINVAL, "repeated site");
        if (a.sorted[0] > a.sorted[1]) { const int t = a.sorted[0]; a.sorted[0] = a.sorted[1]; a.sorted[1] = t; }
    }
    for (int r = 0; r < (1 << k); ++r) a.off[r] = uint32_t(matrix_offset(r, pos, k));
    if (generator) {  // a Pauli product: exactly one nonzero per row
        const int d = 1 << k;
        for (int r = 0; r < d; ++r) {
            int nz = 0;
            for (int c = 0; c < d; ++c) {
                const double re = generator[2 * (r * d + c)], im = generator[2 * (r * d + c) + 1];
                if (re != 0.0 || im != 0.0) {
                    ++nz;
                    a.gcol[r] = c;
                    a.gval[r] = make_double2(re, im);
                }
            }
            if (nz != 1) return set_error(QGB_EINVAL, "generator row %d has %d nonzeros (a Pauli product has one)", r, nz);
        }
    }
    const dim3 grid(unsigned(red_blocks(n)), unsigned(batch));
    double* part = (double*)scratch;
    if (mode == kGradNone) launch_adjoint<kGradNone>(phi, lam, dtype, k, op, a, grid, part, st);
    else if (mode == kGradMatrix) launch_adjoint<kGradMatrix>(phi, lam, dtype, k, op, a, grid, part, st);
    else launch_adjoint<kGradRotation>(phi, lam, dtype, k, op, a, grid, part, st);
    if ((rc = check_launch("adjoint step"))) return rc;
    if (mode == kGradNone) return QGB_OK;
    return finish(part, red_blocks(n), slots, batch, nullptr, grad_out, st);
}

}  // namespace

extern "C" int qgb_adjoint_step_batched(void* phi, void* lam, int dtype, int n, const int* indices, int k,
                                        const void* op, int64_t op_stride, int64_t batch, int64_t sv_stride,
                                        double* grad_out, void* scratch, size_t scratch_bytes, void* stream) {
    return adjoint_impl(phi, lam, dtype, n, indices, k, op, op_stride, batch, sv_stride, nullptr, grad_out, scratch,
                        scratch_bytes, (cudaStream_t)stream);
}

extern "C" int qgb_adjoint_step_rotation(void* phi, void* lam, int dtype, int n, const int* indices, int k,
                                         const void* op, int64_t op_stride, const double* generator, int64_t batch,
                                         int64_t sv_stride, double* grad_out, void* scratch, size_t scratch_bytes,
                                         void* stream) {
    if (!generator || !grad_out) return set_error(QGB_EINVAL, "null generator or output");
    return adjoint_impl(phi, lam, dtype, n, indices, k, op, op_stride, batch, sv_stride, generator, grad_out, scratch,
                        scratch_bytes, (cudaStream_t)stream);
}

extern "C" int qgb_adjoint_step(void* phi, void* lam, int dtype, int n, const int* indices, int k, const void* op,
                                double* grad_out, void* scratch, size_t scratch_bytes, void* stream) {
    return qgb_adjoint_step_batched(phi, lam, dtype, n, indices, k, op, 0, 1, 0, grad_out, scratch, scratch_bytes,
                                    stream);
}

// ---------------------------------------------------------------------------
// Pauli expectation for callers that cannot allocate device memory.
//
// Some callers of this library run where cudaMalloc is off limits: real-time
// loops that must never stall on the allocator, plugins whose host application
// owns all device memory through its own pool and forbids allocations beside
// it, or GPUs whose memory is already fully reserved, where even a small
// allocation fails. qgb_pauli_expectation needs a caller-provided scratch
// buffer for its per-block partial sums; this variant takes its partial sums
// from one fixed array in device memory that is part of the library image
// (1 MiB), so a call allocates nothing -- neither device memory nor host heap
// memory. CUDA loads a library's device code lazily by default, so the array
// is reserved on a device when this file's device code is first loaded there:
// the first call on a device (or the first call of any other reduction entry
// point) reserves it, and it is held until the process exits. A caller that
// reserves all device memory for itself makes one warm-up call first (or sets
// CUDA_MODULE_LOADING=EAGER); the first call on a device also belongs before
// any stream capture. The array's device address is looked up with
// cudaGetSymbolAddress on every call, with the caller's device current: the
// lookup allocates nothing, and a fresh lookup stays right after the context
// is torn down and recreated (cudaDeviceReset), when the module is loaded
// again and the array may move. Every partial-sum slot a call reads was
// written earlier in the same call, so nothing needs clearing between calls;
// but all calls share the one array, so two calls whose kernels overlap on the
// GPU (different streams, or different host threads) race and give wrong
// results.
namespace {

constexpr size_t kNoAllocScratchDoubles = size_t(1) << 17;  // 1 MiB of float64 partial sums
constexpr int kNoAllocMaxTerms = 64;
// red_blocks() never exceeds 1216 partial sums per term, so 64 terms always fit:
// the term count is the only limit
static_assert(size_t(kNoAllocMaxTerms) * 1216 <= kNoAllocScratchDoubles, "fixed scratch too small for 64 terms");

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

void* noalloc_scratch_address(int* rc) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        *rc = set_error(QGB_ECUDA, "cudaGetSymbolAddress of the fixed scratch array: %s", cudaGetErrorString(e));
        return nullptr;
    }
    *rc = QGB_OK;
    return p;
}

}  // namespace

extern "C" int qgb_pauli_expectation_noalloc(const void* sv, int dtype, int n, const char* paulis, const double* coeff,
                                             int nterms, double* out, void* stream) {
    int rc = check_common(sv, dtype, n, 1, 0);
    if (rc) return rc;
    if (!out || !paulis) return set_error(QGB_EINVAL, "null pointer");
    if (n > 64) return set_error(QGB_EINVAL, "Pauli strings limited to 64 sites");
    if (nterms < 1 || nterms > kNoAllocMaxTerms)
        return set_error(QGB_EINVAL, "%d terms requested; the allocation-free variant takes 1..%d (use "
                         "qgb_pauli_expectation for more)", nterms, kNoAllocMaxTerms);
    ParsedPauli ps[kNoAllocMaxTerms];  // parsed on the stack: no heap allocation
    for (int t = 0; t < nterms; ++t) {
        ParsedPauli p{0, 0, 0};
        for (int q = 0; q < n; ++q) {
            const uint64_t bit = 1ull << (n - 1 - q);
            switch (paulis[size_t(t) * n + q]) {
                case 'i': case 'I': break;
                case 'x': case 'X': p.x |= bit; break;
                case 'y': case 'Y': p.x |= bit; p.z |= bit; p.ny++; break;
                case 'z': case 'Z': p.z |= bit; break;
                default: return set_error(QGB_EINVAL, "invalid Pauli character in term %d", t);
            }
        }
        ps[t] = p;
    }
    double* partials = (double*)noalloc_scratch_address(&rc);
    if (!partials) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    int t = 0;
    while (t < nterms) {
        PauliGroup g{};
        g.xmask = ps[t].x;
        g.slot0 = t;
        g.nterms = 0;
        while (t < nterms && ps[t].x == g.xmask && g.nterms < 32) {
            g.zmask[g.nterms] = ps[t].z;
            g.ny[g.nterms] = ps[t].ny;
            g.coeff[g.nterms] = coeff ? coeff[t] : 1.0;
            ++g.nterms;
            ++t;
        }
        if (dtype == QGB_C64) launch_group_nt<float>(sv, n, 0, g, nterms, partials, 1, false, st);
        else launch_group_nt<double>(sv, n, 0, g, nterms, partials, 1, false, st);
        if ((rc = check_launch("pauli expectation (no-alloc)"))) return rc;
    }
    return finish(partials, red_blocks(n), nterms, 1, nullptr, out, st);
}
