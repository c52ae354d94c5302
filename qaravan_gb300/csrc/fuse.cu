// Gate fusion's matrix products on the device.
//
// The fusion compiler (qaravan_gb300/compiler.py) decides on the host which ops
// form each fused block -- pure bookkeeping over bit sets -- and this kernel
// composes the block matrices: block b = E_m ... E_2 E_1, each E the embedding
// of one op's 2^kop x 2^kop matrix into the block's 2^K x 2^K space (op bit j
// on block-matrix bit pos[j], 0 = most significant), applied from the left in
// the ops' order. One CTA per block; the running product lives in shared
// memory in float64 (ping-pong between two 64 KB buffers), the op matrix in a
// third; the result is written in the plan's dtype, row-major, where the
// executor's launches read it. Only the raw op matrices travel from the host.
//
// The reference has no counterpart: it applies every gate as its own pass
// (tensorQ/statevector_sim.py:124-140 via core/base_sim.py:30-53).
//
// Table entries are checked against the block and buffer bounds; an entry
// that fails is skipped and leaves a status word for qgb_check_status.
#include "qgb_common.cuh"

namespace qgb {

__device__ int g_fuse_status = 0;

struct FuseBlock {
    int64_t out;  // element offset of the block's matrix in `out`
    int32_t k, op_begin, op_end, pad;
};

struct FuseEntry {
    int32_t k;
    int32_t pos[QGB_MAX_K];
    int32_t pad;
    int64_t mat;  // complex128 element offset of the op's matrix in `op_mats`
};

static_assert(sizeof(FuseBlock) == 24, "fuse block layout");
static_assert(sizeof(FuseEntry) == 40, "fuse entry layout");

constexpr int kFuseThreads = 256;
constexpr size_t kFuseSmem = 3 * 4096 * sizeof(double2) + 64 * sizeof(int);

template <typename T>
__global__ void __launch_bounds__(kFuseThreads) fuse_blocks_kernel(cplx<T>* __restrict__ out, int64_t out_elems,
                                                                   const FuseBlock* __restrict__ blocks,
                                                                   const FuseEntry* __restrict__ ents, int nents,
                                                                   const double2* __restrict__ op_mats,
                                                                   int64_t op_elems) {
    extern __shared__ __align__(16) unsigned char fuse_smem[];
    double2* M0 = reinterpret_cast<double2*>(fuse_smem);
    double2* M1 = M0 + 4096;
    double2* G = M1 + 4096;
    int* rowbits = reinterpret_cast<int*>(G + 4096);  // block-row bits of each op sub-index
    const FuseBlock B = blocks[blockIdx.x];
    const int K = B.k;
    if (K < 1 || K > QGB_MAX_K || B.op_begin < 0 || B.op_end < B.op_begin || B.op_end > nents || B.out < 0 ||
        B.out + (int64_t(1) << (2 * K)) > out_elems) {
        if (threadIdx.x == 0) atomicExch(&g_fuse_status, 1);
        return;
    }
    const int D = 1 << K;
    for (int i = threadIdx.x; i < D * D; i += kFuseThreads)
        M0[i] = make_double2((i / D) == (i % D) ? 1.0 : 0.0, 0.0);
    for (int e = B.op_begin; e < B.op_end; ++e) {
        const FuseEntry E = ents[e];
        const int kop = E.k;
        bool ok = kop >= 1 && kop <= K && E.mat >= 0 && E.mat + (int64_t(1) << (2 * kop)) <= op_elems;
        int opmask = 0;
        for (int j = 0; ok && j < kop; ++j) {
            const int p = E.pos[j];
            ok = p >= 0 && p < K && !(opmask & (1 << (K - 1 - p)));
            if (ok) opmask |= 1 << (K - 1 - p);
        }
        if (!ok) {  // uniform over the CTA: every thread read the same entry
            if (threadIdx.x == 0) atomicExch(&g_fuse_status, 2);
            continue;
        }
        const int DK = 1 << kop;
        for (int i = threadIdx.x; i < DK * DK; i += kFuseThreads) G[i] = op_mats[E.mat + i];
        for (int s = threadIdx.x; s < DK; s += kFuseThreads) {
            int r = 0;
            for (int j = 0; j < kop; ++j) r |= ((s >> (kop - 1 - j)) & 1) << (K - 1 - E.pos[j]);
            rowbits[s] = r;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < D * D; i += kFuseThreads) {
            const int r = i / D, c = i - (i / D) * D;
            int so = 0;
            for (int j = 0; j < kop; ++j) so |= ((r >> (K - 1 - E.pos[j])) & 1) << (kop - 1 - j);
            const int rbase = r & ~opmask;
            double ax = 0.0, ay = 0.0;
            const double2* grow = G + so * DK;
            for (int si = 0; si < DK; ++si) {
                const double2 g = grow[si], m = M0[(rbase | rowbits[si]) * D + c];
                ax = fma(g.x, m.x, ax);
                ax = fma(-g.y, m.y, ax);
                ay = fma(g.x, m.y, ay);
                ay = fma(g.y, m.x, ay);
            }
            M1[i] = make_double2(ax, ay);
        }
        __syncthreads();
        double2* t = M0;
        M0 = M1;
        M1 = t;
    }
    cplx<T>* o = out + B.out;
    for (int i = threadIdx.x; i < D * D; i += kFuseThreads) o[i] = mk<T>(T(M0[i].x), T(M0[i].y));
}

}  // namespace qgb

using namespace qgb;

namespace qgb_host {

int fuse_status_read_clear() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, qgb::g_fuse_status, sizeof(int)) != cudaSuccess) return -1;
    if (v != 0) {
        const int z = 0;
        cudaMemcpyToSymbol(qgb::g_fuse_status, &z, sizeof(int));
    }
    return v;
}

}  // namespace qgb_host

using namespace qgb_host;

extern "C" size_t qgb_fuse_block_bytes(void) { return sizeof(FuseBlock); }

extern "C" size_t qgb_fuse_entry_bytes(void) { return sizeof(FuseEntry); }

extern "C" int qgb_fuse_blocks(void* out, int dtype, int64_t out_elems, const void* blocks, int nblocks,
                               const void* entries, int nentries, const void* op_mats, int64_t op_elems,
                               void* stream) {
    if (!out || !blocks || (nentries > 0 && (!entries || !op_mats)))
        return set_error(QGB_EINVAL, "null pointer");
    if (nblocks < 0 || nentries < 0 || out_elems < 0 || op_elems < 0) return set_error(QGB_EINVAL, "negative count");
    if (nblocks == 0) return QGB_OK;
    if (nblocks > 2147483647 / 2) return set_error(QGB_EINVAL, "too many blocks");
    const uintptr_t esz = dtype == QGB_C64 ? 8 : 16;
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    if ((reinterpret_cast<uintptr_t>(out) % esz) || (reinterpret_cast<uintptr_t>(op_mats) % 16) ||
        (reinterpret_cast<uintptr_t>(blocks) % 8) || (reinterpret_cast<uintptr_t>(entries) % 8))
        return set_error(QGB_EINVAL, "misaligned table or matrix pointer");
    cudaStream_t st = (cudaStream_t)stream;
    static bool attr[2] = {false, false};
    const int di = dtype == QGB_C64 ? 0 : 1;
    if (!attr[di]) {
        const cudaError_t e = di == 0 ? cudaFuncSetAttribute(fuse_blocks_kernel<float>,
                                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFuseSmem))
                                      : cudaFuncSetAttribute(fuse_blocks_kernel<double>,
                                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFuseSmem));
        if (e != cudaSuccess) return set_error(QGB_ECUDA, "fuse attribute: %s", cudaGetErrorString(e));
        attr[di] = true;
    }
    if (di == 0)
        fuse_blocks_kernel<float><<<nblocks, kFuseThreads, kFuseSmem, st>>>(
            (float2*)out, out_elems, (const FuseBlock*)blocks, (const FuseEntry*)entries, nentries,
            (const double2*)op_mats, op_elems);
    else
        fuse_blocks_kernel<double><<<nblocks, kFuseThreads, kFuseSmem, st>>>(
            (double2*)out, out_elems, (const FuseBlock*)blocks, (const FuseEntry*)entries, nentries,
            (const double2*)op_mats, op_elems);
    return check_launch("fuse blocks");
}
