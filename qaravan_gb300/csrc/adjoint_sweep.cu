// Adjoint reverse sweep with many gates per pass over the state and co-state.
//
// The reference differentiates a circuit through torch autograd, which stores
// every intermediate state (core/param_gates.py:21-49 builds the matrices,
// applications/compilation.py:73-133 calls backward). The adjoint method
// walks the gates backwards carrying phi (the state, uncomputed gate by gate)
// and lam (the co-state); qgb_adjoint_step does one HBM pass over both per
// gate. Here the host groups consecutive gates of the reverse order whose
// sites fit one tile (the geometry of the forward sweeps, sweep.cu): a CTA
// stages the tile of phi and of lam in shared memory (cp.async, double
// buffered), and for every op, in order (consecutive ops on the same sites in
// one register pass),
//   * for a rotation exp(-i theta P) whose derivative is wanted: adds
//     Im sum conj(lam) (P phi) over the tile's groups (float partial per
//     thread, a fixed xor-shuffle tree per warp, a float64 accumulator per
//     (op, warp) in shared memory);
//   * applies U^dagger to both tiles.
// Work is split into chunks of consecutive tiles, each inside one state; a
// chunk's accumulators are summed over the warps in order and stored as one
// partial per (chunk, op), and a second kernel adds the chunks of each state
// in order: bitwise reproducible, no atomics. The scratch size depends on the
// problem only (chunks per state fixed by the batch size).
#include <cstring>

#include "qgb_common.cuh"

namespace qgb {

constexpr int kAdjMaxThreads = 512;
constexpr int kAdjMaxWarps = kAdjMaxThreads / 32;

struct AdjSweepArgs {
    int n, L, H, m, n_ops;
    int high_bits[QGB_SWEEP_MAX_HIGH];
    int n_outer;
    int outer_bits[2 * QGB_MAX_QUBITS];
    int op_k[QGB_SWEEP_MAX_OPS];
    int op_pos[QGB_SWEEP_MAX_OPS][2];
    int64_t op_mat[QGB_SWEEP_MAX_OPS];
    int op_out[QGB_SWEEP_MAX_OPS];
    int gcol[QGB_SWEEP_MAX_OPS][4];
    float2 gval[QGB_SWEEP_MAX_OPS][4];  // entries of a Pauli product: 0, +-1, +-i (exact in float)
    int64_t mat_stride, batch, sv_stride;
    uint64_t tiles;        // tiles per state
    uint64_t chunk_tiles;  // tiles per chunk
    uint64_t chunks;       // chunks over all states
};

__host__ __device__ inline int adj_chunks_per_state(uint64_t tiles, int64_t batch) {
    // ~2048 chunks in all (several per CTA on 152 SMs), a power of two per state
    uint64_t want = 2048 / uint64_t(batch > 0 ? batch : 1);
    uint64_t c = 1;
    while (c * 2 <= want && c * 2 <= tiles) c *= 2;
    return int(c);
}

__device__ __forceinline__ void cp_async16_adj(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(uint32_t(__cvta_generic_to_shared(smem_dst))),
                 "l"(gmem_src)
                 : "memory");
}

constexpr int kAdjMaxRun = 4;  // consecutive ops on the same sites handled in one register pass

// A run of R consecutive ops on the same K sites (R <= kAdjMaxRun): per group
// of partner amplitudes, one load and one store of the staged tiles; for each
// op of the run in order, the derivative (if wanted) at the op's output, then
// U^dagger on both (diagonal ones by one product per amplitude). A single op
// without derivative whose U^dagger permutes (CNOT, SWAP, X) is a copy from the
// permuted tile offsets. threads tid = 0..nthr-1 of the CTA.
template <typename T, int K, int R>
__device__ __forceinline__ void adj_tile_run(cplx<T>* __restrict__ pt, cplx<T>* __restrict__ lt, int m,
                                             const AdjSweepArgs& a, int op0, const cplx<T>* __restrict__ ush,
                                             double* __restrict__ red, int tid, int nthr) {
    constexpr int D = 1 << K;
    using C = cplx<T>;
    int pos[K], srt[K];
#pragma unroll
    for (int j = 0; j < K; ++j) pos[j] = srt[j] = a.op_pos[op0][j];
    if constexpr (K == 2) {
        if (srt[0] > srt[1]) {
            const int t = srt[0];
            srt[0] = srt[1];
            srt[1] = t;
        }
    }
    uint32_t soff[D];
#pragma unroll
    for (int r = 0; r < D; ++r) {
        uint32_t o = 0;
#pragma unroll
        for (int j = 0; j < K; ++j) o |= uint32_t((r >> (K - 1 - j)) & 1) << pos[j];
        soff[r] = swz<T>(o);
    }
    C ud[R][D * D];
    bool want[R];
    C gv[R][D];
    int gc[R][D];
#pragma unroll
    for (int q = 0; q < R; ++q) {
#pragma unroll
        for (int e = 0; e < D * D; ++e) ud[q][e] = ush[(op0 + q) * 16 + e];  // U^dagger, staged per state
        want[q] = a.op_out[op0 + q] >= 0;
#pragma unroll
        for (int r = 0; r < D; ++r) {
            gv[q][r] = mk<T>(T(a.gval[op0 + q][r].x), T(a.gval[op0 + q][r].y));
            gc[q][r] = a.gcol[op0 + q][r];
        }
    }
    // U^dagger diagonal (e.g. RZ, CZ): two complex products per row instead of a row of the matrix
    bool diag[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
        bool d = true;
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int c = 0; c < D; ++c)
                if (r != c) d = d && ud[q][r * D + c].x == T(0) && ud[q][r * D + c].y == T(0);
        diag[q] = d;
    }
    const uint32_t groups = 1u << (m - K);
    if constexpr (R == 1) {
        // a single op without derivative whose U^dagger is a permutation with unit entries
        // (CNOT, SWAP, X): out[r] = in[col(r)], read straight from the permuted tile offsets
        if (!want[0]) {
            int col[D];
            bool perm = true;
#pragma unroll
            for (int r = 0; r < D; ++r) {
                int nz = 0;
                col[r] = 0;
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    const C u = ud[0][r * D + c];
                    if (u.x != T(0) || u.y != T(0)) {
                        ++nz;
                        col[r] = c;
                        perm = perm && u.x == T(1) && u.y == T(0);
                    }
                }
                perm = perm && nz == 1;
            }
            if (perm) {
                uint32_t poff[D];
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    uint32_t o = 0;
#pragma unroll
                    for (int j = 0; j < K; ++j) o |= uint32_t((col[r] >> (K - 1 - j)) & 1) << pos[j];
                    poff[r] = swz<T>(o);
                }
                for (uint32_t g = tid; g < groups; g += nthr) {
                    uint32_t base = g;
#pragma unroll
                    for (int j = 0; j < K; ++j)
                        base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
                    const uint32_t sb = swz<T>(base);
                    C p[D], l[D];
#pragma unroll
                    for (int r = 0; r < D; ++r) {
                        p[r] = pt[sb ^ poff[r]];
                        l[r] = lt[sb ^ poff[r]];
                    }
#pragma unroll
                    for (int r = 0; r < D; ++r) {
                        pt[sb ^ soff[r]] = p[r];
                        lt[sb ^ soff[r]] = l[r];
                    }
                }
                return;
            }
        }
    }
    T s[R];
#pragma unroll
    for (int q = 0; q < R; ++q) s[q] = T(0);
    for (uint32_t g = tid; g < groups; g += nthr) {
        uint32_t base = g;
#pragma unroll
        for (int j = 0; j < K; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
        const uint32_t sb = swz<T>(base);
        C p[D], l[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            p[c] = pt[sb ^ soff[c]];
            l[c] = lt[sb ^ soff[c]];
        }
#pragma unroll
        for (int q = 0; q < R; ++q) {
            if (want[q]) {
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    C pc = p[0];  // p[gc[r]] by selects (no dynamic register indexing)
#pragma unroll
                    for (int c = 1; c < D; ++c)
                        if (gc[q][r] == c) pc = p[c];
                    C w = mk<T>(0, 0);
                    cfma(w, gv[q][r], pc);
                    s[q] += l[r].x * w.y - l[r].y * w.x;  // Im(conj(l) w)
                }
            }
            if (diag[q]) {
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    C x = mk<T>(0, 0), y = mk<T>(0, 0);
                    cfma(x, ud[q][r * D + r], p[r]);
                    cfma(y, ud[q][r * D + r], l[r]);
                    p[r] = x;
                    l[r] = y;
                }
            } else {
                C pn[D], ln[D];
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    C x = mk<T>(0, 0), y = mk<T>(0, 0);
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        cfma(x, ud[q][r * D + c], p[c]);
                        cfma(y, ud[q][r * D + c], l[c]);
                    }
                    pn[r] = x;
                    ln[r] = y;
                }
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    p[r] = pn[r];
                    l[r] = ln[r];
                }
            }
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            pt[sb ^ soff[r]] = p[r];
            lt[sb ^ soff[r]] = l[r];
        }
    }
#pragma unroll
    for (int q = 0; q < R; ++q) {
        if (want[q]) {  // uniform over the CTA: every lane reaches the shuffles
            T v = s[q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if ((tid & 31) == 0) red[(op0 + q) * kAdjMaxWarps + (tid >> 5)] += double(v);
        }
    }
}

// Length of the run of ops starting at op0 on the same sites (same k and tile bits, in order).
__device__ __forceinline__ int adj_run_length(const AdjSweepArgs& a, int op0) {
    int r = 1;
    while (op0 + r < a.n_ops && r < kAdjMaxRun && a.op_k[op0 + r] == a.op_k[op0] &&
           a.op_pos[op0 + r][0] == a.op_pos[op0][0] && (a.op_k[op0] == 1 || a.op_pos[op0 + r][1] == a.op_pos[op0][1]))
        ++r;
    return r;
}

template <typename T, int K>
__device__ __forceinline__ int adj_tile_ops(cplx<T>* pt, cplx<T>* lt, int m, const AdjSweepArgs& a, int op0,
                                            const cplx<T>* ush, double* red, int tid, int nthr) {
    // longest run kept in registers without spilling under the 512-thread register cap
    constexpr int kMax = sizeof(T) == 4 ? (K == 1 ? 4 : 2) : (K == 1 ? 2 : 1);
    int r = adj_run_length(a, op0);
    if (r > kMax) r = kMax;
    if (r == 1) adj_tile_run<T, K, 1>(pt, lt, m, a, op0, ush, red, tid, nthr);
    else if (r == 2) { if constexpr (kMax >= 2) adj_tile_run<T, K, 2>(pt, lt, m, a, op0, ush, red, tid, nthr); }
    else if (r == 3) { if constexpr (kMax >= 3) adj_tile_run<T, K, 3>(pt, lt, m, a, op0, ush, red, tid, nthr); }
    else { if constexpr (kMax >= 4) adj_tile_run<T, K, 4>(pt, lt, m, a, op0, ush, red, tid, nthr); }
    return r;
}

template <typename T>
__global__ void __launch_bounds__(kAdjMaxThreads) adjoint_sweep_kernel(cplx<T>* __restrict__ phi,
                                                                       cplx<T>* __restrict__ lam,
                                                                       const cplx<T>* __restrict__ mats,
                                                                       const __grid_constant__ AdjSweepArgs a,
                                                                       double* __restrict__ partials, int nbuf) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = a.L, H = a.H, m = a.m;
    const int nwarps = blockDim.x >> 5;
    // layout: nbuf x (phi tile, lam tile) | ush (n_ops x 16 complex: U^dagger of the current state) |
    //         hoff (2^H uint64) | red (n_ops x kAdjMaxWarps double)
    C* bufs = reinterpret_cast<C*>(smem_raw);
    C* ush = bufs + (size_t(2 * nbuf) << m);
    uint64_t* hoff = reinterpret_cast<uint64_t*>(ush + size_t(a.n_ops) * 16);
    double* red = reinterpret_cast<double*>(hoff + (size_t(1) << H));
    int64_t staged = -1;  // state whose matrices sit in ush
    for (uint32_t h = threadIdx.x; h < (1u << H); h += blockDim.x) {
        uint64_t o = 0;
        for (int j = 0; j < H; ++j) o |= uint64_t((h >> j) & 1u) << a.high_bits[j];
        hoff[h] = o;
    }
    for (int i = threadIdx.x; i < a.n_ops * kAdjMaxWarps; i += blockDim.x) red[i] = 0.0;
    __syncthreads();
    const uint32_t lmask = (1u << L) - 1;
    constexpr uint32_t per16 = 16 / sizeof(C);
    // this CTA's tiles: chunks blockIdx.x, blockIdx.x + gridDim.x, ..., each chunk_tiles consecutive tiles
    const uint64_t my_chunks = a.chunks > blockIdx.x ? (a.chunks - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint64_t my_tiles = my_chunks * a.chunk_tiles;
    auto tile_of = [&](uint64_t i) -> uint64_t {
        return (uint64_t(blockIdx.x) + (i / a.chunk_tiles) * gridDim.x) * a.chunk_tiles + i % a.chunk_tiles;
    };
    auto base_of = [&](uint64_t w) -> uint64_t {
        const uint64_t b = w / a.tiles, o = w - b * a.tiles;
        uint64_t base = b * uint64_t(a.sv_stride);
        for (int j = 0; j < a.n_outer; ++j) base |= ((o >> j) & 1ull) << a.outer_bits[j];
        return base;
    };
    auto load_async = [&](uint64_t w, C* dp, C* dl) {
        const uint64_t base = base_of(w);
        for (uint32_t e = per16 * threadIdx.x; e < (1u << m); e += per16 * blockDim.x) {
            const uint64_t src = base + (hoff[e >> L] | (e & lmask));
            cp_async16_adj(dp + swz<T>(e), phi + src);
            cp_async16_adj(dl + swz<T>(e), lam + src);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    if (my_tiles > 0) load_async(tile_of(0), bufs, bufs + (size_t(1) << m));
    for (uint64_t i = 0; i < my_tiles; ++i) {
        const uint64_t w = tile_of(i);
        const int slot = nbuf == 2 ? int(i & 1) : 0;
        C* pt = bufs + (size_t(2 * slot) << m);
        C* lt = pt + (size_t(1) << m);
        if (nbuf == 2 && i + 1 < my_tiles) {
            C* np_ = bufs + (size_t(2 * (slot ^ 1)) << m);
            load_async(tile_of(i + 1), np_, np_ + (size_t(1) << m));
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        const int64_t b = int64_t(w / a.tiles);
        if (b != staged) {  // once per chunk: every op's U^dagger for this state (previous readers done: loop-end barrier)
            const C* mb = mats + b * a.mat_stride;
            for (int e = threadIdx.x; e < a.n_ops * 16; e += blockDim.x) {
                const int op = e >> 4, rc = e & 15, d = 1 << a.op_k[op];
                if (rc < d * d) {
                    const int r = rc / d, c = rc - r * d;
                    const C u = mb[a.op_mat[op] + c * d + r];
                    ush[e] = mk<T>(u.x, -u.y);
                }
            }
            staged = b;
        }
        __syncthreads();
        for (int op = 0; op < a.n_ops;) {
            op += a.op_k[op] == 1 ? adj_tile_ops<T, 1>(pt, lt, m, a, op, ush, red, threadIdx.x, blockDim.x)
                                  : adj_tile_ops<T, 2>(pt, lt, m, a, op, ush, red, threadIdx.x, blockDim.x);
            __syncthreads();
        }
        const uint64_t base = base_of(w);
        for (uint32_t e = per16 * threadIdx.x; e < (1u << m); e += per16 * blockDim.x) {
            const uint64_t dst = base + (hoff[e >> L] | (e & lmask));
            *reinterpret_cast<float4*>(phi + dst) = *reinterpret_cast<const float4*>(pt + swz<T>(e));
            *reinterpret_cast<float4*>(lam + dst) = *reinterpret_cast<const float4*>(lt + swz<T>(e));
        }
        if (i % a.chunk_tiles == a.chunk_tiles - 1) {  // chunk done: one partial per op, accumulators reset
            const uint64_t chunk = w / a.chunk_tiles;
            for (int op = threadIdx.x; op < a.n_ops; op += blockDim.x) {
                if (a.op_out[op] < 0) continue;
                double* row = red + op * kAdjMaxWarps;
                double t = 0.0;
                for (int wp = 0; wp < nwarps; ++wp) {
                    t += row[wp];
                    row[wp] = 0.0;
                }
                partials[chunk * a.n_ops + op] = t;
            }
        }
        __syncthreads();  // buffers free for the copy issued next; accumulators reset before the next tile
        if (nbuf == 1 && i + 1 < my_tiles) load_async(tile_of(i + 1), bufs, bufs + (size_t(1) << m));
    }
}

// grad_out[op_out[op] * batch + b] = sum over the state's chunks (in order) of partials[chunk * n_ops + op]
__global__ void adjoint_sweep_finish_kernel(const double* __restrict__ partials, int n_ops, int64_t batch, int cps,
                                            const __grid_constant__ AdjSweepArgs a, double* __restrict__ out) {
    const int64_t item = int64_t(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (item >= batch * n_ops) return;
    const int64_t b = item / n_ops;
    const int op = int(item - b * n_ops);
    if (a.op_out[op] < 0) return;
    double s = 0.0;
    for (int j = lane; j < cps; j += 32) s += partials[(b * cps + j) * n_ops + op];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[int64_t(a.op_out[op]) * batch + b] = s;
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

namespace {

template <typename T>
size_t adj_smem_bytes(int m, int H, int n_ops, int nbuf) {
    return sizeof(cplx<T>) * ((size_t(2 * nbuf) << m) + size_t(n_ops) * 16) + sizeof(uint64_t) * (size_t(1) << H) +
           sizeof(double) * size_t(n_ops) * kAdjMaxWarps;
}

template <typename T>
int launch_adj(void* phi, void* lam, const void* mats, const AdjSweepArgs& a, double* partials, cudaStream_t st) {
    auto kern = adjoint_sweep_kernel<T>;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
            return check_launch("adjoint sweep attribute");
        attr = true;
    }
    for (int nbuf = 2; nbuf >= 1; --nbuf) {
        const size_t smem = adj_smem_bytes<T>(a.m, a.H, a.n_ops, nbuf);
        if (smem > 227 * 1024) continue;
        int per_sm = 0, threads = 256;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem) != cudaSuccess)
            return check_launch("adjoint sweep occupancy");
        if (per_sm < 1) continue;
        if (per_sm == 1) {
            int p512 = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p512, kern, 512, smem) != cudaSuccess)
                return check_launch("adjoint sweep occupancy");
            if (p512 >= 1) threads = 512;
        }
        uint64_t grid = uint64_t(per_sm) * sm_count();
        if (grid > a.chunks) grid = a.chunks;
        kern<<<unsigned(grid), threads, smem, st>>>((cplx<T>*)phi, (cplx<T>*)lam, (const cplx<T>*)mats, a, partials,
                                                    nbuf);
        return check_launch("adjoint sweep kernel");
    }
    return set_error(QGB_EINVAL, "adjoint sweep tile of 2^%d amplitudes does not fit in shared memory", a.m);
}

}  // namespace

extern "C" size_t qgb_adjoint_sweep_scratch_bytes(int n, int tile_bits, int n_ops, int64_t batch) {
    if (n < 1 || n > QGB_MAX_QUBITS || tile_bits < 1 || tile_bits > n || n_ops < 1 || n_ops > QGB_SWEEP_MAX_OPS ||
        batch < 1)
        return 0;
    const uint64_t tiles = uint64_t(1) << (n - tile_bits);
    return sizeof(double) * size_t(batch) * size_t(adj_chunks_per_state(tiles, batch)) * size_t(n_ops);
}

extern "C" int qgb_adjoint_sweep_step(void* phi, void* lam, int dtype, int n, const qgb_adjoint_sweep* sweep,
                                      const void* mats, int64_t mat_stride, int64_t batch, int64_t sv_stride,
                                      double* grad_out, void* scratch, size_t scratch_bytes, void* stream) {
    if (!phi || !lam || !sweep || !mats) return set_error(QGB_EINVAL, "null pointer");
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    if (n < 1 || n > QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "n=%d invalid", n);
    if (batch < 1) return set_error(QGB_EINVAL, "batch %lld < 1", (long long)batch);
    if (batch > 1 && sv_stride < (int64_t(1) << n)) return set_error(QGB_EINVAL, "state stride too small");
    if (mat_stride < 0) return set_error(QGB_EINVAL, "negative matrix stride");
    const int64_t esz = dtype == QGB_C64 ? 8 : 16;
    if ((reinterpret_cast<uintptr_t>(phi) & 15) || (reinterpret_cast<uintptr_t>(lam) & 15) ||
        (batch > 1 && (sv_stride * esz) % 16))
        return set_error(QGB_EINVAL, "state pointers and stride must be 16-byte aligned");
    if (reinterpret_cast<uintptr_t>(mats) % esz) return set_error(QGB_EINVAL, "matrix buffer misaligned");
    const int64_t span = (batch - 1) * (batch > 1 ? sv_stride : 0) + (int64_t(1) << n);
    const char* pb = static_cast<const char*>(phi);
    const char* lb = static_cast<const char*>(lam);
    if (pb < lb + span * esz && lb < pb + span * esz) return set_error(QGB_EINVAL, "the two batches overlap");
    const qgb_adjoint_sweep& sw = *sweep;
    const int L = sw.low_bits, H = sw.n_high, m = L + H;
    if (L < 1 || H < 0 || H > QGB_SWEEP_MAX_HIGH || m > n || m > QGB_SWEEP_MAX_TILE_BITS)
        return set_error(QGB_EINVAL, "tile geometry L=%d H=%d invalid for n=%d", L, H, n);
    if (sw.n_ops < 1 || sw.n_ops > QGB_SWEEP_MAX_OPS) return set_error(QGB_EINVAL, "n_ops=%d out of range", sw.n_ops);
    AdjSweepArgs a{};
    a.n = n;
    a.L = L;
    a.H = H;
    a.m = m;
    a.n_ops = sw.n_ops;
    uint64_t in_tile = (1ull << L) - 1;
    int prev = L - 1;
    for (int h = 0; h < H; ++h) {
        const int b = sw.high_bits[h];
        if (b <= prev || b >= n) return set_error(QGB_EINVAL, "high bits must be ascending, >= L and < n");
        in_tile |= 1ull << b;
        a.high_bits[h] = b;
        prev = b;
    }
    a.n_outer = 0;
    for (int b = 0; b < n; ++b)
        if (!((in_tile >> b) & 1ull)) a.outer_bits[a.n_outer++] = b;
    bool any_out = false;
    for (int i = 0; i < sw.n_ops; ++i) {
        const int k = sw.op_k[i];
        if (k < 1 || k > 2) return set_error(QGB_EINVAL, "adjoint sweep op %d has width %d (1 or 2)", i, k);
        if (k > m) return set_error(QGB_EINVAL, "adjoint sweep op %d wider than the tile", i);
        uint32_t seen = 0;
        for (int j = 0; j < k; ++j) {
            const int p = sw.op_pos[i][j];
            if (p < 0 || p >= m || ((seen >> p) & 1u))
                return set_error(QGB_EINVAL, "adjoint sweep op %d has bad tile bit %d", i, p);
            seen |= 1u << p;
            a.op_pos[i][j] = p;
        }
        if (sw.op_mat[i] < 0) return set_error(QGB_EINVAL, "adjoint sweep op %d has negative matrix offset", i);
        a.op_k[i] = k;
        a.op_mat[i] = sw.op_mat[i];
        a.op_out[i] = sw.op_out[i] < 0 ? -1 : sw.op_out[i];
        if (a.op_out[i] >= 0) {
            any_out = true;
            const int d = 1 << k;
            for (int r = 0; r < d; ++r) {
                const int c = sw.op_gen_col[i][r];
                const double re = sw.op_gen_val[i][r][0], im = sw.op_gen_val[i][r][1];
                const bool unit = (re == 0.0 && (im == 1.0 || im == -1.0)) || (im == 0.0 && (re == 1.0 || re == -1.0));
                if (c < 0 || c >= d || !unit)
                    return set_error(QGB_EINVAL, "adjoint sweep op %d: generator row %d is not a Pauli-product row", i, r);
                a.gcol[i][r] = c;
                a.gval[i][r] = make_float2(float(re), float(im));
            }
        }
    }
    if (any_out && !grad_out) return set_error(QGB_EINVAL, "derivatives requested without an output");
    a.mat_stride = batch > 1 ? mat_stride : 0;
    a.batch = batch;
    a.sv_stride = batch > 1 ? sv_stride : 0;
    a.tiles = uint64_t(1) << (n - m);
    const int cps = adj_chunks_per_state(a.tiles, batch);
    a.chunk_tiles = a.tiles / uint64_t(cps);
    a.chunks = uint64_t(batch) * uint64_t(cps);
    const size_t need = sizeof(double) * size_t(a.chunks) * size_t(a.n_ops);
    if (any_out && (!scratch || scratch_bytes < need))
        return set_error(QGB_ESCRATCH, "scratch of %zu bytes needed (qgb_adjoint_sweep_scratch_bytes)", need);
    cudaStream_t st = (cudaStream_t)stream;
    double* part = (double*)scratch;
    const int rc = dtype == QGB_C64 ? launch_adj<float>(phi, lam, mats, a, part, st)
                                    : launch_adj<double>(phi, lam, mats, a, part, st);
    if (rc || !any_out) return rc;
    const int64_t items = batch * a.n_ops;
    adjoint_sweep_finish_kernel<<<unsigned((items + 7) / 8), 256, 0, st>>>(part, a.n_ops, batch, cps, a, grad_out);
    return check_launch("adjoint sweep finish");
}
