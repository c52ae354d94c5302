// Batched execution of many small, uneven circuits in one launch.
//
// Each CTA owns one circuit whose whole vector (a statevector, or vec(rho) of
// a density matrix, up to 2^14 complex64 / 2^13 complex128 entries) fits in
// shared memory: it loads the vector once, applies the circuit's entire op
// list from a device table (the same swizzled in-tile op code as the sweep
// kernels), and writes it back once -- one HBM round trip per circuit instead
// of one per gate. Circuits of different sizes and depths share the launch;
// the CTA count is the number of circuits.
#include "sweep_common.cuh"

namespace qgb {

struct BatchCircuit {
    int64_t offset;      // element offset of the vector in the state buffer
    int64_t out_offset;  // double offset of this circuit's results in `out` (epilogue)
    int32_t nbits;       // vector of 2^nbits entries
    int32_t op_begin, op_end;
    int32_t flags;       // bit 0: start from the basis state 0 instead of loading the vector
    int32_t dm_sites;    // > 0: vector is vec(rho) of dm_sites qubits; write trace, purity, <Z_i>
    int32_t pad;
};

struct BatchOp {
    int32_t k;
    int32_t pos[QGB_MAX_K];  // flat bit positions, matrix order
    int64_t mat;             // element offset of the matrix
};

constexpr int kMaxDmSites = 7;

template <typename T, int KMAX>
__global__ void __launch_bounds__(512) batch_small_kernel(cplx<T>* __restrict__ states, const BatchCircuit* __restrict__ circs,
                                                          const BatchOp* __restrict__ ops, const cplx<T>* __restrict__ mats,
                                                          double* __restrict__ out, int max_bits) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const BatchCircuit c = circs[blockIdx.x];
    const int m = c.nbits;
    if (m < 1 || m > max_bits) return;  // larger than the staged buffer: the host never emits it
    C* tile = reinterpret_cast<C*>(smem_raw);
    C* msh = tile + (size_t(1) << m);
    C* s = states + c.offset;
    if (c.flags & 1) {
        for (uint32_t e = threadIdx.x; e < (1u << m); e += blockDim.x) tile[swz<T>(e)] = mk<T>(e == 0 ? T(1) : T(0), T(0));
    } else {
        for (uint32_t e = threadIdx.x; e < (1u << m); e += blockDim.x) tile[swz<T>(e)] = s[e];
    }
    __syncthreads();
    for (int i = c.op_begin; i < c.op_end; ++i) {
        const BatchOp op = ops[i];
        // ops outside the vector's bits are skipped (the host never emits them)
        bool valid = op.k >= 1 && op.k <= KMAX && op.k <= m;
        uint32_t seen = 0;
        for (int j = 0; j < op.k && j < QGB_MAX_K; ++j) {
            valid = valid && op.pos[j] >= 0 && op.pos[j] < m && !((seen >> op.pos[j]) & 1u);
            if (valid) seen |= 1u << op.pos[j];
        }
        if (!valid) continue;
        const C* mat = mats + op.mat;
        if (op.k == 1) tile_op<T, 1, CtaSync>(tile, m, op.pos, mat, msh, threadIdx.x, blockDim.x);
        else if (op.k == 2) { if constexpr (KMAX >= 2) tile_op<T, 2, CtaSync>(tile, m, op.pos, mat, msh, threadIdx.x, blockDim.x); }
        else if (op.k == 3) { if constexpr (KMAX >= 3) tile_op<T, 3, CtaSync>(tile, m, op.pos, mat, msh, threadIdx.x, blockDim.x); }
        else if (op.k == 4) { if constexpr (KMAX >= 4) tile_op<T, 4, CtaSync>(tile, m, op.pos, mat, msh, threadIdx.x, blockDim.x); }
        __syncthreads();
    }
    for (uint32_t e = threadIdx.x; e < (1u << m); e += blockDim.x) s[e] = tile[swz<T>(e)];
    if (out != nullptr && c.dm_sites > 0 && c.dm_sites <= kMaxDmSites && 2 * c.dm_sites == m) {
        // epilogue on the staged vec(rho): Re Tr(rho), Tr(rho^2) = sum |rho_xy|^2, Re Tr(rho Z_i), in float64
        const int nq = c.dm_sites;
        double acc[2 + kMaxDmSites];
        for (int j = 0; j < 2 + kMaxDmSites; ++j) acc[j] = 0.0;
        for (uint32_t e = threadIdx.x; e < (1u << m); e += blockDim.x) {
            const C v = tile[swz<T>(e)];
            acc[1] += double(v.x) * v.x + double(v.y) * v.y;
            const uint32_t x = e >> nq, y = e & ((1u << nq) - 1);
            if (x == y) {
                acc[0] += double(v.x);
                for (int q = 0; q < nq; ++q) acc[2 + q] += ((x >> (nq - 1 - q)) & 1u) ? -double(v.x) : double(v.x);
            }
        }
        __shared__ double red[16][2 + kMaxDmSites];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int j = 0; j < 2 + nq; ++j) {
            double v = acc[j];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) red[warp][j] = v;
        }
        __syncthreads();
        if (threadIdx.x < 2 + nq) {
            double v = 0;
            for (int w = 0; w < int(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
            out[c.out_offset + threadIdx.x] = v;
        }
    }
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

namespace {

template <typename T, int KMAX>
int launch_small(void* states, const void* circs, int ncirc, const void* ops, const void* mats, int max_bits,
                 double* out, cudaStream_t st) {
    const size_t smem = sizeof(cplx<T>) * ((size_t(1) << max_bits) + stage_elems<KMAX>());
    auto kern = batch_small_kernel<T, KMAX>;
    static size_t dyn_max = 0;
    if (dyn_max == 0) {
        // the epilogue's reduction buffer is static shared memory: opt in to the rest
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) return check_launch("batch attributes");
        dyn_max = 227 * 1024 - fa.sharedSizeBytes;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dyn_max)) != cudaSuccess) {
            dyn_max = 0;
            return check_launch("batch attribute");
        }
    }
    if (smem > dyn_max) return set_error(QGB_EINVAL, "vectors of 2^%d entries do not fit in shared memory", max_bits);
    const int threads = max_bits >= 12 ? 512 : 256;
    kern<<<unsigned(ncirc), threads, smem, st>>>((cplx<T>*)states, (const BatchCircuit*)circs, (const BatchOp*)ops,
                                                 (const cplx<T>*)mats, out, max_bits);
    return check_launch("batch kernel");
}

}  // namespace

extern "C" size_t qgb_batch_circuit_bytes(void) { return sizeof(BatchCircuit); }
extern "C" size_t qgb_batch_op_bytes(void) { return sizeof(BatchOp); }

extern "C" int qgb_batch_small(void* states, int dtype, const void* circuits, int ncirc, const void* ops,
                               const void* mats, int max_bits, int max_k, double* out, void* stream) {
    if (!states || !circuits || !ops || !mats) return set_error(QGB_EINVAL, "null pointer");
    if (ncirc < 1 || ncirc > 1 << 20) return set_error(QGB_EINVAL, "circuit count %d out of range", ncirc);
    if (max_bits < 1 || max_bits > (dtype == QGB_C64 ? 14 : 13))
        return set_error(QGB_EINVAL, "vectors of 2^%d entries do not fit in shared memory", max_bits);
    if (max_k < 1 || max_k > 4 || max_k > max_bits) return set_error(QGB_EINVAL, "op width %d unsupported (1..4)", max_k);
    cudaStream_t st = (cudaStream_t)stream;
    const int km = max_k < 2 ? 2 : max_k;
    if (dtype == QGB_C64) {
        switch (km) {
            case 2: return launch_small<float, 2>(states, circuits, ncirc, ops, mats, max_bits, out, st);
            case 3: return launch_small<float, 3>(states, circuits, ncirc, ops, mats, max_bits, out, st);
            case 4: return launch_small<float, 4>(states, circuits, ncirc, ops, mats, max_bits, out, st);
        }
    } else if (dtype == QGB_C128) {
        switch (km) {
            case 2: return launch_small<double, 2>(states, circuits, ncirc, ops, mats, max_bits, out, st);
            case 3: return launch_small<double, 3>(states, circuits, ncirc, ops, mats, max_bits, out, st);
            case 4: return launch_small<double, 4>(states, circuits, ncirc, ops, mats, max_bits, out, st);
        }
    }
    return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
}
