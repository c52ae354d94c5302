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

// ---- packed fp32x2 arithmetic (one instruction = two FMAs) ----------------
__device__ __forceinline__ uint64_t pack2(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(__float_as_uint(lo)), "r"(__float_as_uint(hi)));
    return r;
}
__device__ __forceinline__ uint64_t swap2(uint64_t v) {
    uint32_t lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(v));
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(hi), "r"(lo));
    return r;
}
__device__ __forceinline__ uint64_t ffma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Applies one dense op of width K to the whole tile. `tile` is swizzled with
// swz<T>, which is linear over XOR, so swz(base | off) = swz(base) ^ swz(off)
// and the per-access address costs one XOR.
template <typename T, int K>
__device__ __forceinline__ void tile_op(cplx<T>* __restrict__ tile, int m, const int* pos_in,
                                        const cplx<T>* __restrict__ mat, cplx<T>* __restrict__ msh) {
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
    if constexpr (K <= 2 && sizeof(T) == 4) {
        // complex MAC as two packed FMAs: acc += (m.x, m.x) * (v.x, v.y) + (-m.y, m.y) * (v.y, v.x)
        uint64_t A1[D * D], A2[D * D];
#pragma unroll
        for (int i = 0; i < D * D; ++i) {
            const float2 mm = __ldg(reinterpret_cast<const float2*>(mat) + i);
            A1[i] = pack2(mm.x, mm.x);
            A2[i] = pack2(-mm.y, mm.y);
        }
        uint64_t* t64 = reinterpret_cast<uint64_t*>(tile);
        for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
            uint32_t base = g;
#pragma unroll
            for (int j = 0; j < K; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
            const uint32_t sb = swz<T>(base);
            uint64_t v[D], vs[D];
#pragma unroll
            for (int c = 0; c < D; ++c) {
                v[c] = t64[sb ^ soff[c]];
                vs[c] = swap2(v[c]);
            }
#pragma unroll
            for (int r = 0; r < D; ++r) {
                uint64_t acc = 0;
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    acc = ffma2(A1[r * D + c], v[c], acc);
                    acc = ffma2(A2[r * D + c], vs[c], acc);
                }
                t64[sb ^ soff[r]] = acc;
            }
        }
    } else if constexpr (K <= 2) {
        C mr[D * D];
#pragma unroll
        for (int i = 0; i < D * D; ++i) mr[i] = __ldg(&mat[i]);
        for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
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
        const C* mm = mat;
        if constexpr (K <= kStageK) {
            for (int i = threadIdx.x; i < D * D; i += blockDim.x) msh[i] = mat[i];
            __syncthreads();
            mm = msh;
        }
        for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
            uint32_t base = g;
#pragma unroll
            for (int j = 0; j < K; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
            const uint32_t sb = swz<T>(base);
            C v[D];
#pragma unroll
            for (int c = 0; c < D; ++c) v[c] = tile[sb ^ soff[c]];
#pragma unroll 1
            for (int r = 0; r < D; ++r) {
                const C* mrow = mm + r * D;
                C acc = mk<T>(0, 0);
#pragma unroll
                for (int c = 0; c < D; ++c) cfma(acc, mrow[c], v[c]);
                uint32_t o = 0;
#pragma unroll
                for (int j = 0; j < K; ++j) o |= uint32_t((r >> (K - 1 - j)) & 1) << pos[j];
                tile[sb ^ swz<T>(o)] = acc;
            }
        }
    }
}

// All ops of a sweep on one staged tile, with a CTA barrier after each op.
template <typename T, int KMAX>
__device__ __forceinline__ void apply_ops(cplx<T>* tile, int m, const SweepArgs& a, const cplx<T>* mb, cplx<T>* msh) {
    for (int i = 0; i < a.sw.n_ops; ++i) {
        const int k = a.sw.op_k[i];
        const cplx<T>* mat = mb + a.sw.op_mat[i];
        const int* pos = a.sw.op_pos[i];
        if (k == 1) tile_op<T, 1>(tile, m, pos, mat, msh);
        else if (k == 2) { if constexpr (KMAX >= 2) tile_op<T, 2>(tile, m, pos, mat, msh); }
        else if (k == 3) { if constexpr (KMAX >= 3) tile_op<T, 3>(tile, m, pos, mat, msh); }
        else if (k == 4) { if constexpr (KMAX >= 4) tile_op<T, 4>(tile, m, pos, mat, msh); }
        else if (k == 5) { if constexpr (KMAX >= 5) tile_op<T, 5>(tile, m, pos, mat, msh); }
        __syncthreads();
    }
}

}  // namespace qgb

namespace qgb_host {
// TMA-staged double-buffered sweep (sweep_tma.cu). Returns 1 if the geometry
// is not eligible (caller falls back to the load/store kernel), else a QGB code.
int launch_sweep_tma(int dtype, void* sv, const void* mats, const qgb::SweepArgs& a, int kmax, cudaStream_t st);
int sweep_status_read_clear();
}  // namespace qgb_host
