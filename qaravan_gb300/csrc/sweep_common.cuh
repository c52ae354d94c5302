// Shared pieces of the two sweep kernels: launch arguments and the in-tile
// dense op (a 2^k x 2^k matrix applied to every group of partner amplitudes
// of a tile staged in shared memory).
#pragma once

#include "qgb_common.cuh"

namespace qgb {

struct SweepArgs {
    qgb_sweep sw;
    int n;  // bits per vector
    int n_outer;
    int outer_bits[2 * QGB_MAX_QUBITS];
    int64_t mat_stride, batch, sv_stride;
    uint64_t tiles;  // tiles per vector
};

constexpr int kStageK = 4;  // ops with 3 <= k <= 4 stage their matrix in shared memory

template <int KMAX> __host__ __device__ constexpr int stage_elems() { return KMAX >= 3 ? (1 << (2 * (KMAX < kStageK ? KMAX : kStageK))) : 0; }

// Barrier over the threads that run the ops: the whole CTA, or (in the
// warp-specialised kernel) only the compute warps, on named barrier 1.
struct CtaSync {
    __device__ static void sync(int) { __syncthreads(); }
};
struct ComputeSync {
    __device__ static void sync(int nthr) { asm volatile("bar.sync 1, %0;" ::"r"(nthr) : "memory"); }
};

// Applies one dense op of width K to the whole tile, threads tid = 0..nthr-1.
// `tile` is swizzled with swz<T>, which is linear over XOR, so
// swz(base | off) = swz(base) ^ swz(off) and each access costs one XOR.
template <typename T, int K, typename Sync>
__device__ __forceinline__ void tile_op(cplx<T>* __restrict__ tile, int m, const int* pos_in,
                                        const cplx<T>* __restrict__ mat, cplx<T>* __restrict__ msh, int tid,
                                        int nthr) {
    constexpr int D = 1 << K;
    using C = cplx<T>;
    int pos[K], srt[K];
#pragma unroll
    for (int j = 0; j < K; ++j) pos[j] = srt[j] = pos_in[j];
#pragma unroll
    for (int i = 1; i < K; ++i)
#pragma unroll
        for (int j = i; j > 0; --j)
            if (srt[j - 1] > srt[j]) {
                int t = srt[j];
                srt[j] = srt[j - 1];
                srt[j - 1] = t;
            }
    uint32_t soff[D];
#pragma unroll
    for (int r = 0; r < D; ++r) {
        uint32_t o = 0;
#pragma unroll
        for (int j = 0; j < K; ++j) o |= uint32_t((r >> (K - 1 - j)) & 1) << pos[j];
        soff[r] = swz<T>(o);
    }
    const uint32_t groups = 1u << (m - K);
    if constexpr (K <= 2) {
        C mr[D * D];
#pragma unroll
        for (int i = 0; i < D * D; ++i) mr[i] = __ldg(&mat[i]);
        for (uint32_t g = tid; g < groups; g += nthr) {
            uint32_t base = g;
#pragma unroll
            for (int j = 0; j < K; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
            const uint32_t sb = swz<T>(base);
            C v[D];
#pragma unroll
            for (int c = 0; c < D; ++c) v[c] = tile[sb ^ soff[c]];
#pragma unroll
            for (int r = 0; r < D; ++r) {
                C acc = mk<T>(0, 0);
#pragma unroll
                for (int c = 0; c < D; ++c) cfma(acc, mr[r * D + c], v[c]);
                tile[sb ^ soff[r]] = acc;
            }
        }
    } else {
        // Wide op: the matrix is read from shared memory (staged for K <= 4),
        // two element pairs per 16-byte load, and every element feeds two groups.
        const C* mm = mat;
        if constexpr (K <= kStageK) {
            for (int i = tid; i < D * D; i += nthr) msh[i] = mat[i];
            Sync::sync(nthr);
            mm = msh;
        }
        // groups g and g + half go together (a single group is processed twice when the op spans the tile)
        const uint32_t half = groups > 1 ? groups >> 1 : 1;
        for (uint32_t g = tid; g < half; g += nthr) {
            uint32_t b0 = g, b1 = groups > 1 ? g + half : g;
#pragma unroll
            for (int j = 0; j < K; ++j) {
                b0 = ((b0 >> srt[j]) << (srt[j] + 1)) | (b0 & ((1u << srt[j]) - 1));
                b1 = ((b1 >> srt[j]) << (srt[j] + 1)) | (b1 & ((1u << srt[j]) - 1));
            }
            const uint32_t s0 = swz<T>(b0), s1 = swz<T>(b1);
            C v0[D], v1[D];
#pragma unroll
            for (int c = 0; c < D; ++c) {
                v0[c] = tile[s0 ^ soff[c]];
                v1[c] = tile[s1 ^ soff[c]];
            }
#pragma unroll 1
            for (int r = 0; r < D; ++r) {
                const C* mrow = mm + r * D;
                C a0 = mk<T>(0, 0), a1 = mk<T>(0, 0);
                if constexpr (sizeof(T) == 4) {
                    const float4* m4 = reinterpret_cast<const float4*>(mrow);
#pragma unroll
                    for (int c = 0; c < D; c += 2) {
                        const float4 q = m4[c >> 1];
                        const C e0 = mk<T>(q.x, q.y), e1 = mk<T>(q.z, q.w);
                        cfma(a0, e0, v0[c]);
                        cfma(a1, e0, v1[c]);
                        cfma(a0, e1, v0[c + 1]);
                        cfma(a1, e1, v1[c + 1]);
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        const C e = mrow[c];
                        cfma(a0, e, v0[c]);
                        cfma(a1, e, v1[c]);
                    }
                }
                uint32_t o = 0;
#pragma unroll
                for (int j = 0; j < K; ++j) o |= uint32_t((r >> (K - 1 - j)) & 1) << pos[j];
                const uint32_t so = swz<T>(o);
                tile[s0 ^ so] = a0;
                tile[s1 ^ so] = a1;
            }
        }
    }
}

// All ops of a sweep on one staged tile, with a barrier after each op.
template <typename T, int KMAX, typename Sync>
__device__ __forceinline__ void apply_ops(cplx<T>* tile, int m, const SweepArgs& a, const cplx<T>* mb, cplx<T>* msh,
                                          int tid, int nthr) {
    for (int i = 0; i < a.sw.n_ops; ++i) {
        const int k = a.sw.op_k[i];
        const cplx<T>* mat = mb + a.sw.op_mat[i];
        const int* pos = a.sw.op_pos[i];
        if (k == 1) tile_op<T, 1, Sync>(tile, m, pos, mat, msh, tid, nthr);
        else if (k == 2) { if constexpr (KMAX >= 2) tile_op<T, 2, Sync>(tile, m, pos, mat, msh, tid, nthr); }
        else if (k == 3) { if constexpr (KMAX >= 3) tile_op<T, 3, Sync>(tile, m, pos, mat, msh, tid, nthr); }
        else if (k == 4) { if constexpr (KMAX >= 4) tile_op<T, 4, Sync>(tile, m, pos, mat, msh, tid, nthr); }
        else if (k == 5) { if constexpr (KMAX >= 5) tile_op<T, 5, Sync>(tile, m, pos, mat, msh, tid, nthr); }
        Sync::sync(nthr);
    }
}

}  // namespace qgb

namespace qgb_host {
// TMA-staged double-buffered sweep (sweep_tma.cu). Returns 1 if the geometry
// is not eligible (caller falls back to the load/store kernel), else a QGB code.
int launch_sweep_tma(int dtype, void* sv, const void* mats, const qgb::SweepArgs& a, int kmax, cudaStream_t st);
int sweep_status_read_clear();
// complex128 tile sweeps in double-float arithmetic (sweep_df.cu); c128_arith() is
// 1 when they are selected (the default), 0 for the float64 kernels.
int c128_arith();
int launch_sweep_df(void* sv, const void* mats, const qgb::SweepArgs& a, int kmax, cudaStream_t st);
}  // namespace qgb_host
