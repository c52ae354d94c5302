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
//     thread, a fixed xor-shuffle tree per warp, a compensated float
//     accumulator per (op, warp) in shared memory -- float64 for complex128);
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
    // register runs: consecutive ops on at most `rbits` tile bits, applied to groups of
    // 2^rbits amplitudes of both tiles held in registers (0: one shared-memory pass per op)
    int rbits;
    int run_len[QGB_SWEEP_MAX_OPS];     // at a run's first op: its op count (0 elsewhere)
    int run_pos[QGB_SWEEP_MAX_OPS][4];  // at a run's first op: the tile bit of each local bit of the run
    int op_lpos[QGB_SWEEP_MAX_OPS][2];  // every op's sites as local bits of its run
    int op_gcls[QGB_SWEEP_MAX_OPS];     // generator class of a wanted derivative (kGenNone: none)
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
                                             typename WAccOf<T>::type* __restrict__ red, int tid, int nthr) {
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
            if ((tid & 31) == 0) wacc_add(red[(op0 + q) * kAdjMaxWarps + (tid >> 5)], v);
        }
    }
}

// ---- register runs -------------------------------------------------------
// An op of a run acts on a group of 2^R amplitudes of phi and lam held in
// registers; local bit P of the group <-> tile bit run_pos[P]. Positions are
// runtime values: each (R, positions) case is its own fully unrolled instance,
// chosen by a switch. For each op: the derivative (if wanted) at the op's
// output, Im sum_r conj(l_r) (gval_r p_{gcol_r}), then U^dagger on both --
// dense, diagonal (two products per row) or a permutation with unit entries
// (register moves), as classified when the state's matrices were staged.
constexpr int kAdjDense = 0, kAdjDiag = 1, kAdjPerm = 2, kAdjReal = 3;  // kAdjReal: a dense real matrix (RY)
// permutations of a two-site U^dagger known at compile time (register renaming, no selects):
// rows (0, 1, 2, 3) <- columns (0, 1, 3, 2) [CNOT, control on the first site], (0, 3, 2, 1)
// [CNOT, control on the second site], (0, 2, 1, 3) [SWAP]
constexpr int kAdjPermCX = 4, kAdjPermXC = 5, kAdjPermSwap = 6;
// generator classes of a wanted derivative (host-classified Pauli-product rows): none, diagonal
// (row r reads column r), flipped (one site: row r reads r ^ 1; two sites: 3 - r), any other
constexpr int kGenNone = 0, kGenDiag = 1, kGenFlip = 2, kGenAny = 3;

// The derivative Im sum_r conj(l_r) (g_r p_{col r}) of one op over a group: complex sums
// W_r = sum conj(l_r) q_r per generator row r, combined once per op as Im(g_r W_r) =
// g_r.x W_r.y + g_r.y W_r.x (g_r in {+-1, +-i}).
template <typename T, typename C>
__device__ __forceinline__ void wacc(C& w, const C& l, const C& q) {
    w.x = fmaf(l.x, q.x, fmaf(l.y, q.y, w.x));
    w.y = fmaf(l.x, q.y, fmaf(-l.y, q.x, w.y));
}
template <>
__device__ __forceinline__ void wacc<double, double2>(double2& w, const double2& l, const double2& q) {
    w.x = fma(l.x, q.x, fma(l.y, q.y, w.x));
    w.y = fma(l.x, q.y, fma(-l.y, q.x, w.y));
}

template <int R, int P, int MODE, int GEN, typename C, typename T>
__device__ __forceinline__ void adj_reg1(C (&p)[1 << R], C (&l)[1 << R], const C* __restrict__ u,
                                         const float2* gv, T& s) {
    constexpr int D = 1 << R, bit = 1 << P;
    const C u0 = u[0], u1 = u[1], u2 = u[2], u3 = u[3];
    C w0 = mk<T>(T(0), T(0)), w1 = mk<T>(T(0), T(0));
#pragma unroll
    for (int c = 0; c < D; ++c) {
        if (c & bit) continue;
        const C p0 = p[c], p1 = p[c | bit], l0 = l[c], l1 = l[c | bit];
        if constexpr (GEN == kGenDiag) {
            wacc<T>(w0, l0, p0);
            wacc<T>(w1, l1, p1);
        } else if constexpr (GEN != kGenNone) {  // one site: off-diagonal rows (X, Y)
            wacc<T>(w0, l0, p1);
            wacc<T>(w1, l1, p0);
        }
        if constexpr (MODE == kAdjReal) {
            const T a = u0.x, b = u1.x, cc = u2.x, d = u3.x;
            p[c] = mk<T>(a * p0.x + b * p1.x, a * p0.y + b * p1.y);
            p[c | bit] = mk<T>(cc * p0.x + d * p1.x, cc * p0.y + d * p1.y);
            l[c] = mk<T>(a * l0.x + b * l1.x, a * l0.y + b * l1.y);
            l[c | bit] = mk<T>(cc * l0.x + d * l1.x, cc * l0.y + d * l1.y);
        } else if constexpr (MODE == kAdjDiag) {
            C x = mk<T>(0, 0), y = mk<T>(0, 0), z = mk<T>(0, 0), t = mk<T>(0, 0);
            cfma(x, u0, p0);
            cfma(y, u3, p1);
            cfma(z, u0, l0);
            cfma(t, u3, l1);
            p[c] = x;
            p[c | bit] = y;
            l[c] = z;
            l[c | bit] = t;
        } else if constexpr (MODE == kAdjPerm) {  // one site: a unit permutation that is not the identity swaps
            p[c] = p1;
            p[c | bit] = p0;
            l[c] = l1;
            l[c | bit] = l0;
        } else {
            C x = mk<T>(0, 0), y = mk<T>(0, 0), z = mk<T>(0, 0), t = mk<T>(0, 0);
            cfma(x, u0, p0);
            cfma(x, u1, p1);
            cfma(y, u2, p0);
            cfma(y, u3, p1);
            cfma(z, u0, l0);
            cfma(z, u1, l1);
            cfma(t, u2, l0);
            cfma(t, u3, l1);
            p[c] = x;
            p[c | bit] = y;
            l[c] = z;
            l[c | bit] = t;
        }
    }
    if constexpr (GEN != kGenNone)
        s += T(gv[0].x) * w0.y + T(gv[0].y) * w0.x + T(gv[1].x) * w1.y + T(gv[1].y) * w1.x;
}

// matrix bit 1 (most significant) <-> local bit P0 (the op's first site), bit 0 <-> P1
template <int R, int P0, int P1, int MODE, int GEN, typename C, typename T>
__device__ __forceinline__ void adj_reg2(C (&p)[1 << R], C (&l)[1 << R], const C* __restrict__ u,
                                         const uint8_t* __restrict__ col, const float2* gv, const int* gc, T& s) {
    constexpr int D = 1 << R, b0 = 1 << P0, b1 = 1 << P1;
    int gcr[4], colr[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        gcr[r] = GEN == kGenAny ? gc[r] : 0;
        colr[r] = MODE == kAdjPerm ? col[r] : 0;
    }
    C w[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) w[r] = mk<T>(T(0), T(0));
#pragma unroll
    for (int c = 0; c < D; ++c) {
        if ((c & b0) || (c & b1)) continue;
        const int ix[4] = {c, c | b1, c | b0, c | b0 | b1};
        C x[4], y[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            x[r] = p[ix[r]];
            y[r] = l[ix[r]];
        }
        if constexpr (GEN == kGenDiag) {
#pragma unroll
            for (int r = 0; r < 4; ++r) wacc<T>(w[r], y[r], x[r]);
        } else if constexpr (GEN == kGenFlip) {
#pragma unroll
            for (int r = 0; r < 4; ++r) wacc<T>(w[r], y[r], x[3 - r]);
        } else if constexpr (GEN == kGenAny) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                C q = x[0];  // x[gc[r]] by selects (no dynamic register indexing)
#pragma unroll
                for (int e = 1; e < 4; ++e)
                    if (gcr[r] == e) q = x[e];
                wacc<T>(w[r], y[r], q);
            }
        }
        if constexpr (MODE == kAdjDiag) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const C d = u[5 * r];
                C a = mk<T>(0, 0), b = mk<T>(0, 0);
                cfma(a, d, x[r]);
                cfma(b, d, y[r]);
                p[ix[r]] = a;
                l[ix[r]] = b;
            }
        } else if constexpr (MODE == kAdjPermCX || MODE == kAdjPermXC || MODE == kAdjPermSwap) {
            constexpr int s1 = MODE == kAdjPermCX ? 1 : (MODE == kAdjPermXC ? 3 : 2);
            constexpr int s2 = MODE == kAdjPermCX ? 3 : (MODE == kAdjPermXC ? 2 : 1);
            constexpr int s3 = MODE == kAdjPermCX ? 2 : (MODE == kAdjPermXC ? 1 : 3);
            p[ix[1]] = x[s1];
            p[ix[2]] = x[s2];
            p[ix[3]] = x[s3];
            l[ix[1]] = y[s1];
            l[ix[2]] = y[s2];
            l[ix[3]] = y[s3];
        } else if constexpr (MODE == kAdjPerm) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                C a = x[0], b = y[0];
#pragma unroll
                for (int e = 1; e < 4; ++e)
                    if (colr[r] == e) {
                        a = x[e];
                        b = y[e];
                    }
                p[ix[r]] = a;
                l[ix[r]] = b;
            }
        } else {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                C a = mk<T>(0, 0), b = mk<T>(0, 0);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const C m = u[4 * r + e];
                    cfma(a, m, x[e]);
                    cfma(b, m, y[e]);
                }
                p[ix[r]] = a;
                l[ix[r]] = b;
            }
        }
    }
    if constexpr (GEN != kGenNone) {
#pragma unroll
        for (int r = 0; r < 4; ++r) s += T(gv[r].x) * w[r].y + T(gv[r].y) * w[r].x;
    }
}

// the op's class and generator class, chosen once per op (each case its own unrolled code)
template <int R, int P, int GEN, typename C, typename T>
__device__ __forceinline__ void adj_reg1_mode(C (&p)[1 << R], C (&l)[1 << R], const C* u, int mode, const float2* gv,
                                              T& s) {
    switch (mode) {
        case kAdjReal: adj_reg1<R, P, kAdjReal, GEN>(p, l, u, gv, s); break;
        case kAdjDiag: adj_reg1<R, P, kAdjDiag, GEN>(p, l, u, gv, s); break;
        case kAdjPerm: adj_reg1<R, P, kAdjPerm, GEN>(p, l, u, gv, s); break;
        default: adj_reg1<R, P, kAdjDense, GEN>(p, l, u, gv, s); break;
    }
}

template <int R, int P, typename C, typename T>
__device__ __forceinline__ void adj_reg1_any(C (&p)[1 << R], C (&l)[1 << R], const C* u, int mode, int gen,
                                             const float2* gv, T& s) {
    switch (gen) {
        case kGenNone: adj_reg1_mode<R, P, kGenNone>(p, l, u, mode, gv, s); break;
        case kGenDiag: adj_reg1_mode<R, P, kGenDiag>(p, l, u, mode, gv, s); break;
        default: adj_reg1_mode<R, P, kGenFlip>(p, l, u, mode, gv, s); break;
    }
}

template <int R, int P0, int P1, int GEN, typename C, typename T>
__device__ __forceinline__ void adj_reg2_mode(C (&p)[1 << R], C (&l)[1 << R], const C* u, int mode,
                                              const uint8_t* col, const float2* gv, const int* gc, T& s) {
    switch (mode) {
        case kAdjDiag: adj_reg2<R, P0, P1, kAdjDiag, GEN>(p, l, u, col, gv, gc, s); break;
        case kAdjPermCX: adj_reg2<R, P0, P1, kAdjPermCX, GEN>(p, l, u, col, gv, gc, s); break;
        case kAdjPermXC: adj_reg2<R, P0, P1, kAdjPermXC, GEN>(p, l, u, col, gv, gc, s); break;
        case kAdjPermSwap: adj_reg2<R, P0, P1, kAdjPermSwap, GEN>(p, l, u, col, gv, gc, s); break;
        case kAdjPerm: adj_reg2<R, P0, P1, kAdjPerm, GEN>(p, l, u, col, gv, gc, s); break;
        default: adj_reg2<R, P0, P1, kAdjDense, GEN>(p, l, u, col, gv, gc, s); break;
    }
}

template <int R, int P0, int P1, typename C, typename T>
__device__ __forceinline__ void adj_reg2_any(C (&p)[1 << R], C (&l)[1 << R], const C* u, int mode, int gen,
                                             const uint8_t* col, const float2* gv, const int* gc, T& s) {
    switch (gen) {
        case kGenNone: adj_reg2_mode<R, P0, P1, kGenNone>(p, l, u, mode, col, gv, gc, s); break;
        case kGenDiag: adj_reg2_mode<R, P0, P1, kGenDiag>(p, l, u, mode, col, gv, gc, s); break;
        case kGenFlip: adj_reg2_mode<R, P0, P1, kGenFlip>(p, l, u, mode, col, gv, gc, s); break;
        default: adj_reg2_mode<R, P0, P1, kGenAny>(p, l, u, mode, col, gv, gc, s); break;
    }
}

template <int R, typename C, typename T>
__device__ __forceinline__ void adj_apply1(C (&p)[1 << R], C (&l)[1 << R], int P, const C* u, int mode, int gen,
                                           const float2* gv, T& s) {
    switch (P) {
        case 0: adj_reg1_any<R, 0>(p, l, u, mode, gen, gv, s); break;
        case 1: if constexpr (R > 1) adj_reg1_any<R, 1>(p, l, u, mode, gen, gv, s); break;
        case 2: if constexpr (R > 2) adj_reg1_any<R, 2>(p, l, u, mode, gen, gv, s); break;
        case 3: if constexpr (R > 3) adj_reg1_any<R, 3>(p, l, u, mode, gen, gv, s); break;
    }
}

template <int R, int CODE, typename C, typename T>
__device__ __forceinline__ void adj_apply2_case(C (&p)[1 << R], C (&l)[1 << R], const C* u, int mode, int gen,
                                                const uint8_t* col, const float2* gv, const int* gc, T& s) {
    constexpr int P0 = CODE / 4, P1 = CODE % 4;
    if constexpr (P0 < R && P1 < R && P0 != P1) adj_reg2_any<R, P0, P1>(p, l, u, mode, gen, col, gv, gc, s);
}

template <int R, typename C, typename T>
__device__ __forceinline__ void adj_apply2(C (&p)[1 << R], C (&l)[1 << R], int P0, int P1, const C* u, int mode,
                                           int gen, const uint8_t* col, const float2* gv, const int* gc, T& s) {
    switch (P0 * 4 + P1) {
        case 1: adj_apply2_case<R, 1>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 2: adj_apply2_case<R, 2>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 3: adj_apply2_case<R, 3>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 4: adj_apply2_case<R, 4>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 6: adj_apply2_case<R, 6>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 7: adj_apply2_case<R, 7>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 8: adj_apply2_case<R, 8>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 9: adj_apply2_case<R, 9>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 11: adj_apply2_case<R, 11>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 12: adj_apply2_case<R, 12>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 13: adj_apply2_case<R, 13>(p, l, u, mode, gen, col, gv, gc, s); break;
        case 14: adj_apply2_case<R, 14>(p, l, u, mode, gen, col, gv, gc, s); break;
    }
}

// Every run of the pass on one staged pair of tiles: groups of 2^R amplitudes,
// one group per thread at a time, a barrier after each run. umode / ucol: each
// op's U^dagger class and, for a permutation, its source column per row.
template <typename T, int R>
__device__ __forceinline__ void adj_tile_runs(cplx<T>* __restrict__ pt, cplx<T>* __restrict__ lt, int m,
                                              const AdjSweepArgs& a, const cplx<T>* __restrict__ ush,
                                              const uint8_t* __restrict__ umode, const uint8_t* __restrict__ ucol,
                                              typename WAccOf<T>::type* __restrict__ red, int tid, int nthr) {
    using C = cplx<T>;
    constexpr int D = 1 << R;
    const int warp = tid >> 5, lane = tid & 31;
    for (int i0 = 0; i0 < a.n_ops;) {
        const int nr = a.run_len[i0];
        int rp[R], srt[R];
#pragma unroll
        for (int j = 0; j < R; ++j) rp[j] = srt[j] = a.run_pos[i0][j];
#pragma unroll
        for (int x = 1; x < R; ++x)
#pragma unroll
            for (int y = x; y > 0; --y)
                if (srt[y - 1] > srt[y]) {
                    const int t = srt[y];
                    srt[y] = srt[y - 1];
                    srt[y - 1] = t;
                }
        uint32_t soff[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            uint32_t o = 0;
#pragma unroll
            for (int j = 0; j < R; ++j) o |= uint32_t((c >> j) & 1) << rp[j];
            soff[c] = swz<T>(o);
        }
        const uint32_t groups = 1u << (m - R);
        for (uint32_t gb = 0; gb < groups; gb += uint32_t(nthr)) {  // every thread the same trip count
            const uint32_t g = gb + uint32_t(tid);
            const bool ok = g < groups;
            uint32_t base = ok ? g : 0u;
#pragma unroll
            for (int j = 0; j < R; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
            const uint32_t sb = swz<T>(base);
            C p[D], l[D];
#pragma unroll
            for (int c = 0; c < D; ++c) {
                p[c] = ok ? pt[sb ^ soff[c]] : mk<T>(T(0), T(0));
                l[c] = ok ? lt[sb ^ soff[c]] : mk<T>(T(0), T(0));
            }
            for (int q = 0; q < nr; ++q) {
                const int op = i0 + q;
                const int gen = a.op_gcls[op];
                const bool want = gen != kGenNone;
                T sd = T(0);
                if (a.op_k[op] == 1)
                    adj_apply1<R>(p, l, a.op_lpos[op][0], ush + op * 16, umode[op], gen, a.gval[op], sd);
                else
                    adj_apply2<R>(p, l, a.op_lpos[op][0], a.op_lpos[op][1], ush + op * 16, umode[op], gen,
                                  ucol + op * 4, a.gval[op], a.gcol[op], sd);
                if (want) {  // uniform over the CTA: every lane reaches the shuffles
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, o);
                    if (lane == 0) wacc_add(red[op * kAdjMaxWarps + warp], sd);
                }
            }
            if (ok) {
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    pt[sb ^ soff[c]] = p[c];
                    lt[sb ^ soff[c]] = l[c];
                }
            }
        }
        __syncthreads();
        i0 += nr;
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
                                            const cplx<T>* ush, typename WAccOf<T>::type* red, int tid, int nthr) {
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

// complex64: 256 threads and 3 CTAs per SM (80 registers): the passes are latency-bound, and
// the third CTA's warps outweigh the few register spills (64-set, 20-qubit gradient 0.42 ->
// 0.36 s); complex128 keeps 128 registers (up to 512 threads when one CTA fits)
template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 256 : kAdjMaxThreads, sizeof(T) == 4 ? 3 : 1) adjoint_sweep_kernel(cplx<T>* __restrict__ phi,
                                                                       cplx<T>* __restrict__ lam,
                                                                       const cplx<T>* __restrict__ mats,
                                                                       const __grid_constant__ AdjSweepArgs a,
                                                                       double* __restrict__ partials, int nbuf) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = a.L, H = a.H, m = a.m;
    const int nwarps = blockDim.x >> 5;
    // layout: nbuf x (phi tile, lam tile) | ush (n_ops x 16 complex: U^dagger of the current state) |
    //         hoff (2^H uint64) | red (n_ops x kAdjMaxWarps accumulators, 8 bytes) | umode (n_ops) | ucol (n_ops x 4)
    C* bufs = reinterpret_cast<C*>(smem_raw);
    C* ush = bufs + (size_t(2 * nbuf) << m);
    uint64_t* hoff = reinterpret_cast<uint64_t*>(ush + size_t(a.n_ops) * 16);
    auto* red = reinterpret_cast<typename WAccOf<T>::type*>(hoff + (size_t(1) << H));
    uint8_t* umode = reinterpret_cast<uint8_t*>(red + size_t(a.n_ops) * kAdjMaxWarps);
    uint8_t* ucol = umode + a.n_ops;
    int64_t staged = -1;  // state whose matrices sit in ush
    for (uint32_t h = threadIdx.x; h < (1u << H); h += blockDim.x) {
        uint64_t o = 0;
        for (int j = 0; j < H; ++j) o |= uint64_t((h >> j) & 1u) << a.high_bits[j];
        hoff[h] = o;
    }
    for (int i = threadIdx.x; i < a.n_ops * kAdjMaxWarps; i += blockDim.x) wacc_zero(red[i]);
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
            if (a.rbits > 0) {
                __syncthreads();
                // classify each op's U^dagger: diagonal, a permutation with unit entries, or dense
                for (int op = threadIdx.x; op < a.n_ops; op += blockDim.x) {
                    const int d = 1 << a.op_k[op];
                    const C* u = ush + op * 16;
                    bool diag = true, perm = true, real = true;
                    for (int r = 0; r < d; ++r) {
                        int nz = 0, cc = 0;
                        for (int c = 0; c < d; ++c) {
                            const C v = u[r * d + c];
                            const bool z = v.x == T(0) && v.y == T(0);
                            if (v.y != T(0)) real = false;
                            if (r != c && !z) diag = false;
                            if (!z) {
                                ++nz;
                                cc = c;
                                perm = perm && v.x == T(1) && v.y == T(0);
                            }
                        }
                        perm = perm && nz == 1;
                        ucol[op * 4 + r] = uint8_t(cc);
                    }
                    int mode = diag ? kAdjDiag : (perm ? kAdjPerm : ((real && d == 2) ? kAdjReal : kAdjDense));
                    if (mode == kAdjPerm && d == 4) {
                        const uint8_t* c4 = ucol + op * 4;
                        if (c4[0] == 0 && c4[1] == 1 && c4[2] == 3 && c4[3] == 2) mode = kAdjPermCX;
                        else if (c4[0] == 0 && c4[1] == 3 && c4[2] == 2 && c4[3] == 1) mode = kAdjPermXC;
                        else if (c4[0] == 0 && c4[1] == 2 && c4[2] == 1 && c4[3] == 3) mode = kAdjPermSwap;
                    }
                    umode[op] = uint8_t(mode);
                }
            }
            staged = b;
        }
        __syncthreads();
        if (a.rbits == 3) {
            adj_tile_runs<T, 3>(pt, lt, m, a, ush, umode, ucol, red, threadIdx.x, blockDim.x);
        } else {
            for (int op = 0; op < a.n_ops;) {
                op += a.op_k[op] == 1 ? adj_tile_ops<T, 1>(pt, lt, m, a, op, ush, red, threadIdx.x, blockDim.x)
                                      : adj_tile_ops<T, 2>(pt, lt, m, a, op, ush, red, threadIdx.x, blockDim.x);
                __syncthreads();
            }
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
                auto* row = red + op * kAdjMaxWarps;
                double t = 0.0;
                for (int wp = 0; wp < nwarps; ++wp) {
                    t += wacc_value(row[wp]);
                    wacc_zero(row[wp]);
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
           sizeof(double) * size_t(n_ops) * kAdjMaxWarps + size_t(n_ops) * 5;
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
        if (per_sm == 1 && sizeof(T) == 8) {
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

int g_adj_run_bits = -1;  // register runs: -1 default (on), 0 per-op passes

// Register runs span 3 tile bits (8-amplitude groups of both tiles); 16-amplitude
// groups measured slower (more registers and code per op) and are not built.
int adj_run_bits(int dtype) {
    (void)dtype;
    return g_adj_run_bits == 0 ? 0 : 3;
}

}  // namespace

extern "C" int qgb_set_adjoint_runs(int bits) {
    if (bits != -1 && bits != 0 && bits != 3)
        return set_error(QGB_EINVAL, "adjoint register-run width %d (-1 default, 0 off, 3)", bits);
    g_adj_run_bits = bits;
    return QGB_OK;
}

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
        a.op_gcls[i] = kGenNone;
        if (a.op_out[i] >= 0) {
            any_out = true;
            const int d = 1 << k;
            uint32_t cols = 0;
            bool gdiag = true, gflip = true;
            for (int r = 0; r < d; ++r) {
                const int c = sw.op_gen_col[i][r];
                const double re = sw.op_gen_val[i][r][0], im = sw.op_gen_val[i][r][1];
                const bool unit = (re == 0.0 && (im == 1.0 || im == -1.0)) || (im == 0.0 && (re == 1.0 || re == -1.0));
                if (c < 0 || c >= d || !unit)
                    return set_error(QGB_EINVAL, "adjoint sweep op %d: generator row %d is not a Pauli-product row", i, r);
                a.gcol[i][r] = c;
                a.gval[i][r] = make_float2(float(re), float(im));
                cols |= 1u << c;
                gdiag = gdiag && c == r;
                gflip = gflip && c == d - 1 - r;
            }
            if (cols != (1u << d) - 1u)
                return set_error(QGB_EINVAL, "adjoint sweep op %d: generator rows are not a permutation", i);
            a.op_gcls[i] = gdiag ? kGenDiag : (gflip ? kGenFlip : kGenAny);
        }
    }
    if (any_out && !grad_out) return set_error(QGB_EINVAL, "derivatives requested without an output");
    // register runs: greedy, consecutive ops while their sites fit rbits tile bits
    a.rbits = adj_run_bits(dtype);
    if (a.rbits > m) a.rbits = m;
    if (a.rbits >= 3) {
        for (int i0 = 0; i0 < sw.n_ops;) {
            uint32_t bits = 0;
            int i = i0;
            for (; i < sw.n_ops; ++i) {
                uint32_t nb = bits;
                for (int j = 0; j < a.op_k[i]; ++j) nb |= 1u << a.op_pos[i][j];
                if (__builtin_popcount(nb) > a.rbits) break;
                bits = nb;
            }
            // the run's local bits: its own tile bits ascending, then the lowest unused ones
            int nrp = 0;
            for (int b = 0; b < m && nrp < a.rbits; ++b)
                if ((bits >> b) & 1u) a.run_pos[i0][nrp++] = b;
            for (int b = 0; b < m && nrp < a.rbits; ++b)
                if (!((bits >> b) & 1u)) a.run_pos[i0][nrp++] = b;
            a.run_len[i0] = i - i0;
            for (int o = i0; o < i; ++o)
                for (int j = 0; j < a.op_k[o]; ++j)
                    for (int r = 0; r < a.rbits; ++r)
                        if (a.run_pos[i0][r] == a.op_pos[o][j]) a.op_lpos[o][j] = r;
            i0 = i;
        }
    } else {
        a.rbits = 0;
    }
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
