// Noisy trajectories in one persistent launch.
//
// The reference samples noisy circuits one at a time on the CPU (MonteCarloSim,
// tensorQ/monte_carlo_sim.py:14-35, one statevector run per sample). Here one
// launch runs every trajectory through the whole circuit:
//
//  * each CTA takes the next trajectory from a work counter (an atomic ticket,
//    nobody waits on anybody) and owns it to the end: the circuit is cut on the
//    host into tile sweeps (ops whose bits fit one shared-memory tile: the low
//    L bits times H chosen high bits), and the CTA streams the trajectory's
//    state through shared memory once per sweep -- cp.async double buffering,
//    every op of the sweep applied to the staged tile -- ping-ponging between
//    the trajectory's own slot and a per-CTA scratch vector;
//  * after every gate, on each of its sites, a depolarising channel (I, or X,
//    Y, Z with p/3 each, sampled from Philox with the same counters as the
//    gate-by-gate kernel, so both paths draw the same Paulis) and amplitude
//    damping (Kraus K0 = diag(1, sqrt(1 - gamma)), K1 = sqrt(gamma) |0><1|);
//  * amplitude damping is unravelled exactly by the no-jump norm: the state
//    is advanced with K0 unnormalised; its squared norm after channel m,
//    N_m = N_{m-1} - gamma W_m (W_m the weight of the site's |1> component
//    just before the channel), is the probability of no jump up to m; with a
//    uniform threshold r the first jump is at the first m with N_m < r, which
//    has probability N_{m-1} - N_m = gamma W_m, as the sequential rule. The
//    W_m of a sweep are summed over its tiles; at the sweep's end the CTA walks
//    the channels, and if a jump falls inside the sweep it runs the sweep again
//    from its (untouched) input with K1 at that channel, renormalised, and a
//    fresh threshold. Without a jump the threshold carries over as r / N_end
//    (the conditional law) and the next sweep's first op rescales the state by
//    1 / sqrt(N_end). A last pass writes the normalised state to the
//    trajectory's slot.
//
// Random numbers: Philox4x32-10 (philox.cuh). Pauli of site j after gate g:
// counter (g, trajectory, 2j, 0), as the gate-by-gate kernel; jump threshold
// number i of a trajectory: counter (i, trajectory, 0, 2).
#include "philox.cuh"
#include "qgb_common.cuh"

namespace qgb {

using TrajSweepDesc = qgb_traj_sweep;
using TrajOpDesc = qgb_traj_op;

constexpr int kTrajMaxOps = 128;    // ops per sweep
constexpr int kTrajMaxJumps = 16;   // jumps inside one sweep of one trajectory
constexpr int kTrajThreads = 512;  // 16 warps, one register group each at a time (98 registers): 15 % faster than
                                    // 8 warps with two groups each (215 registers), the latency-bound runs

struct TrajRunArgs {
    int n;
    int64_t ntraj, stride;
    int nsweeps;
    double p_dep, gamma;
    uint32_t seed0, seed1;
    int nbuf;            // tile buffers (2: the next tile's copy overlaps the ops)
    int mmax;            // largest tile bits of any sweep
    int max_log;         // jump log entries per trajectory
};

__device__ int g_traj_status = 0;

__device__ __forceinline__ void traj_cp16(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(uint32_t(__cvta_generic_to_shared(smem_dst))),
                 "l"(gmem_src)
                 : "memory");
}

template <typename T> __device__ __forceinline__ uint32_t tswz(uint32_t e);
template <> __device__ __forceinline__ uint32_t tswz<float>(uint32_t e) { return swz<float>(e); }
template <> __device__ __forceinline__ uint32_t tswz<double>(uint32_t e) { return swz<double>(e); }

// ---- ops on a register group ------------------------------------------------
// A run of consecutive ops whose sites lie within R tile bits is applied to
// groups of 2^R amplitudes held in registers: local index bit P <-> the run's
// tile position run_pos[P]. Positions are runtime values; each (width,
// positions) case is its own fully unrolled instance, chosen by a switch, so
// the group never leaves registers.

template <typename C> __device__ __forceinline__ C cmul(const C& a, const C& b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

template <int R, int P, typename C>
__device__ __forceinline__ void reg_op1(C (&v)[1 << R], const C* __restrict__ m, bool diag) {
    constexpr int D = 1 << R, bit = 1 << P;
    const C m00 = m[0], m01 = m[1], m10 = m[2], m11 = m[3];
    if (diag) {
#pragma unroll
        for (int c = 0; c < D; ++c) v[c] = cmul(v[c], (c & bit) ? m11 : m00);
        return;
    }
#pragma unroll
    for (int c = 0; c < D; ++c) {
        if (c & bit) continue;
        const C a = v[c], b = v[c | bit];
        C x = cmul(m00, a), y = cmul(m10, a);
        cfma(x, m01, b);
        cfma(y, m11, b);
        v[c] = x;
        v[c | bit] = y;
    }
}

// matrix index bit 1 (most significant) <-> local position P0 (the op's first site), bit 0 <-> P1
template <int R, int P0, int P1, typename C>
__device__ __forceinline__ void reg_op2(C (&v)[1 << R], const C* __restrict__ m, bool diag) {
    constexpr int D = 1 << R, b0 = 1 << P0, b1 = 1 << P1;
    if (diag) {
        const C d0 = m[0], d1 = m[5], d2 = m[10], d3 = m[15];
#pragma unroll
        for (int c = 0; c < D; ++c) v[c] = cmul(v[c], (c & b0) ? ((c & b1) ? d3 : d2) : ((c & b1) ? d1 : d0));
        return;
    }
    C mm[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) mm[e] = m[e];
#pragma unroll
    for (int c = 0; c < D; ++c) {
        if ((c & b0) || (c & b1)) continue;
        const C x[4] = {v[c], v[c | b1], v[c | b0], v[c | b0 | b1]};
        C y[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            y[r] = cmul(mm[4 * r], x[0]);
#pragma unroll
            for (int k = 1; k < 4; ++k) cfma(y[r], mm[4 * r + k], x[k]);
        }
        v[c] = y[0];
        v[c | b1] = y[1];
        v[c | b0] = y[2];
        v[c | b0 | b1] = y[3];
    }
}

// Amplitude damping of the site at local position P: w += weight of its |1>
// components; then K0 (mode 1: |1> components times s0) or the jump (mode 2:
// the |1> components times sj move to |0>, |1> cleared).
template <int R, int P, typename C, typename T>
__device__ __forceinline__ void reg_damp(C (&v)[1 << R], int mode, T s0, T sj, T& w) {
    constexpr int D = 1 << R, bit = 1 << P;
#pragma unroll
    for (int c = 0; c < D; ++c) {
        if (!(c & bit)) continue;
        w = fma(v[c].x, v[c].x, w);
        w = fma(v[c].y, v[c].y, w);
        if (mode == 1) {
            v[c].x *= s0;
            v[c].y *= s0;
        } else {
            v[c ^ bit].x = sj * v[c].x;
            v[c ^ bit].y = sj * v[c].y;
            v[c].x = T(0);
            v[c].y = T(0);
        }
    }
}

template <int R, typename C>
__device__ __forceinline__ void reg_apply1(C (&v)[1 << R], int P, const C* m, bool diag) {
    switch (P) {
        case 0: reg_op1<R, 0>(v, m, diag); break;
        case 1: if constexpr (R > 1) reg_op1<R, 1>(v, m, diag); break;
        case 2: if constexpr (R > 2) reg_op1<R, 2>(v, m, diag); break;
        case 3: if constexpr (R > 3) reg_op1<R, 3>(v, m, diag); break;
    }
}

template <int R, int CODE, typename C>
__device__ __forceinline__ void reg_apply2_case(C (&v)[1 << R], const C* m, bool diag) {
    constexpr int P0 = CODE / 4, P1 = CODE % 4;
    if constexpr (P0 < R && P1 < R && P0 != P1) reg_op2<R, P0, P1>(v, m, diag);
}

template <int R, typename C>
__device__ __forceinline__ void reg_apply2(C (&v)[1 << R], int P0, int P1, const C* m, bool diag) {
    switch (P0 * 4 + P1) {
        case 1: reg_apply2_case<R, 1>(v, m, diag); break;
        case 2: reg_apply2_case<R, 2>(v, m, diag); break;
        case 3: reg_apply2_case<R, 3>(v, m, diag); break;
        case 4: reg_apply2_case<R, 4>(v, m, diag); break;
        case 6: reg_apply2_case<R, 6>(v, m, diag); break;
        case 7: reg_apply2_case<R, 7>(v, m, diag); break;
        case 8: reg_apply2_case<R, 8>(v, m, diag); break;
        case 9: reg_apply2_case<R, 9>(v, m, diag); break;
        case 11: reg_apply2_case<R, 11>(v, m, diag); break;
        case 12: reg_apply2_case<R, 12>(v, m, diag); break;
        case 13: reg_apply2_case<R, 13>(v, m, diag); break;
        case 14: reg_apply2_case<R, 14>(v, m, diag); break;
    }
}

template <int R, typename C, typename T>
__device__ __forceinline__ void reg_damp_at(C (&v)[1 << R], int P, int mode, T s0, T sj, T& w) {
    switch (P) {
        case 0: reg_damp<R, 0>(v, mode, s0, sj, w); break;
        case 1: if constexpr (R > 1) reg_damp<R, 1>(v, mode, s0, sj, w); break;
        case 2: if constexpr (R > 2) reg_damp<R, 2>(v, mode, s0, sj, w); break;
        case 3: if constexpr (R > 3) reg_damp<R, 3>(v, mode, s0, sj, w); break;
    }
}

// Per-warp accumulators of the damping weights (WAccOf, qgb_common.cuh): for
// complex64 a compensated float sum -- a float64 add per warp, op and tile kept
// GB300's narrow FP64 pipe 38 % busy -- for complex128 a double.
// Per-sweep, per-trajectory state in dynamic shared memory.
template <typename T> struct TrajSweepSmem {
    cplx<T>* msh;     // [op][16]: the op's matrix with its sampled Paulis folded in (first op: times the prescale)
    typename WAccOf<T>::type* chw_w;  // [warp][2 * kTrajMaxOps]: per-warp weights of |1> before each damping
    T* djump;         // [op][2]: jump factor sqrt(gamma) / sqrt(gamma W) where a jump is replayed
    uint8_t* dmode;   // [op][2]: 0 none, 1 K0, 2 jump
    uint8_t* dflag;   // [op]: the folded matrix is diagonal
};

// Every run of a sweep on one staged tile; G groups of 2^R amplitudes per
// thread at a time, a barrier after each run.
template <typename T, int R, int G>
__device__ __forceinline__ void traj_tile_runs(cplx<T>* __restrict__ tile, int m, const TrajOpDesc* __restrict__ ops,
                                               int nops, const TrajSweepSmem<T>& sm, bool damp, T s0, int tid,
                                               int nthr) {
    using C = cplx<T>;
    constexpr int D = 1 << R;
    const int warp = tid >> 5, lane = tid & 31;
    auto* myw = sm.chw_w + size_t(warp) * (2 * kTrajMaxOps);
    for (int i0 = 0; i0 < nops;) {
        const int nr = ops[i0].run;
        int rp[R], srt[R];
#pragma unroll
        for (int j = 0; j < R; ++j) rp[j] = srt[j] = ops[i0].run_pos[j];
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
        for (int l = 0; l < D; ++l) {
            uint32_t o = 0;
#pragma unroll
            for (int j = 0; j < R; ++j) o |= uint32_t((l >> j) & 1) << rp[j];
            soff[l] = tswz<T>(o);
        }
        const uint32_t groups = 1u << (m - R);
        for (uint32_t gb = 0; gb < groups; gb += uint32_t(G * nthr)) {
            C v[G][D];
            uint32_t sb[G];
            bool ok[G];
#pragma unroll
            for (int gi = 0; gi < G; ++gi) {
                const uint32_t g = gb + uint32_t(gi * nthr + tid);
                ok[gi] = g < groups;
                uint32_t base = ok[gi] ? g : 0u;
#pragma unroll
                for (int j = 0; j < R; ++j)
                    base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
                sb[gi] = tswz<T>(base);
#pragma unroll
                for (int l = 0; l < D; ++l) v[gi][l] = ok[gi] ? tile[sb[gi] ^ soff[l]] : mk<T>(T(0), T(0));
            }
            for (int q = 0; q < nr; ++q) {
                const int i = i0 + q;
                const int k = ops[i].k, p0 = ops[i].lpos[0], p1 = ops[i].lpos[1];
                const C* mm = sm.msh + size_t(i) * 16;
                const bool dg = sm.dflag[i] != 0;
                T w0 = T(0), w1 = T(0);  // the state's precision: the jump and renormalisation factors come from these
#pragma unroll
                for (int gi = 0; gi < G; ++gi) {
                    if (k == 1) reg_apply1<R>(v[gi], p0, mm, dg);
                    else reg_apply2<R>(v[gi], p0, p1, mm, dg);
                }
                if (damp) {
                    const int d0 = sm.dmode[2 * i], d1 = sm.dmode[2 * i + 1];
                    const T j0 = sm.djump[2 * i], j1 = sm.djump[2 * i + 1];
#pragma unroll
                    for (int gi = 0; gi < G; ++gi) {
                        reg_damp_at<R>(v[gi], p0, d0, s0, j0, w0);
                        if (k == 2) reg_damp_at<R>(v[gi], p1, d1, s0, j1, w1);
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        w0 += __shfl_xor_sync(0xffffffffu, w0, o);
                        w1 += __shfl_xor_sync(0xffffffffu, w1, o);
                    }
                    if (lane == 0) {
                        wacc_add(myw[2 * i], w0);
                        wacc_add(myw[2 * i + 1], w1);
                    }
                }
            }
#pragma unroll
            for (int gi = 0; gi < G; ++gi)
                if (ok[gi])
#pragma unroll
                    for (int l = 0; l < D; ++l) tile[sb[gi] ^ soff[l]] = v[gi][l];
        }
        __syncthreads();
        i0 += nr;
    }
}

template <typename T, int RMAX>
__device__ __forceinline__ void traj_tile_dispatch(cplx<T>* tile, int m, const TrajOpDesc* ops, int nops,
                                                   const TrajSweepSmem<T>& sm, bool damp, T s0, int tid, int nthr) {
    const int R = m < RMAX ? m : RMAX;
    switch (R) {
        case 1: traj_tile_runs<T, 1, 1>(tile, m, ops, nops, sm, damp, s0, tid, nthr); break;
        case 2: traj_tile_runs<T, 2, 1>(tile, m, ops, nops, sm, damp, s0, tid, nthr); break;
        case 3: traj_tile_runs<T, 3, 1>(tile, m, ops, nops, sm, damp, s0, tid, nthr); break;
        default: if constexpr (RMAX >= 4) traj_tile_runs<T, 4, 1>(tile, m, ops, nops, sm, damp, s0, tid, nthr); break;
    }
}

template <typename T> constexpr int traj_rmax() { return sizeof(T) == 4 ? 4 : 3; }

// dynamic shared memory: tile buffers | high-bit offsets | folded matrices | per-warp weights | jump factors |
// damping modes | diagonal flags
template <typename T> __host__ __device__ constexpr size_t traj_aux_bytes() {
    return sizeof(uint32_t) * (size_t(1) << QGB_SWEEP_MAX_HIGH) + sizeof(cplx<T>) * kTrajMaxOps * 16 +
           sizeof(typename WAccOf<T>::type) * (kTrajThreads / 32) * 2 * kTrajMaxOps + sizeof(T) * 2 * kTrajMaxOps +
           2 * kTrajMaxOps +
           kTrajMaxOps;
}

template <typename T>
__global__ void __launch_bounds__(kTrajThreads) traj_run_kernel(cplx<T>* __restrict__ states,
                                                                cplx<T>* __restrict__ pingpong,
                                                                const TrajSweepDesc* __restrict__ sweeps,
                                                                const TrajOpDesc* __restrict__ ops,
                                                                const cplx<T>* __restrict__ mats, int* queue,
                                                                int* __restrict__ jump_count, int* __restrict__ jump_log,
                                                                const __grid_constant__ TrajRunArgs a) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char traj_smem[];
    C* bufs = reinterpret_cast<C*>(traj_smem);
    uint32_t* hoff = reinterpret_cast<uint32_t*>(bufs + (size_t(a.nbuf) << a.mmax));
    TrajSweepSmem<T> sm;
    sm.msh = reinterpret_cast<C*>(hoff + (size_t(1) << QGB_SWEEP_MAX_HIGH));
    sm.chw_w = reinterpret_cast<typename WAccOf<T>::type*>(sm.msh + kTrajMaxOps * 16);
    sm.djump = reinterpret_cast<T*>(sm.chw_w + (kTrajThreads / 32) * 2 * kTrajMaxOps);
    sm.dmode = reinterpret_cast<uint8_t*>(sm.djump + 2 * kTrajMaxOps);
    sm.dflag = sm.dmode + 2 * kTrajMaxOps;
    __shared__ double chw[2 * kTrajMaxOps];  // per (op, site): weight of |1> before damping, summed over the tiles
    __shared__ uint8_t pk[kTrajMaxOps][2];   // sampled Paulis
    __shared__ int jop[kTrajMaxJumps], jsite[kTrajMaxJumps];
    __shared__ double jscale[kTrajMaxJumps];
    __shared__ int s_traj, s_njump, s_replay;
    __shared__ double s_r, s_prescale;
    __shared__ int s_jumps_total;
    const int tid = threadIdx.x, nthr = blockDim.x, nwarps = blockDim.x >> 5;
    const uint64_t dim = uint64_t(1) << a.n;
    C* scratch = pingpong + uint64_t(blockIdx.x) * dim;
    const T s0 = T(sqrt(1.0 - a.gamma));
    const bool damp = a.gamma > 0;
    constexpr uint32_t per16 = 16 / sizeof(C);
    while (true) {
        if (tid == 0) {
            s_traj = atomicAdd(queue, 1);
            s_r = Philox::uniform4(0u, uint32_t(s_traj), 0u, 2u, a.seed0, a.seed1);
            s_prescale = 1.0;
            s_jumps_total = 0;
        }
        __syncthreads();
        const int64_t t = s_traj;
        if (t >= a.ntraj) break;
        C* own = states + t * a.stride;
        C* src = nullptr;  // null: the sweep starts from |0...0>
        C* dst = scratch;
        for (int s = 0; s < a.nsweeps; ++s) {
            const TrajSweepDesc sw = sweeps[s];
            const int L = sw.L, H = sw.H, m = L + H, nops = sw.op_end - sw.op_begin;
            const TrajOpDesc* sops = ops + sw.op_begin;
            const uint32_t lmask = (1u << L) - 1u;
            // tile-index -> global offset of the high bits; the outer bits enumerate tiles
            for (uint32_t h = tid; h < (1u << H); h += nthr) {
                uint32_t o = 0;
                for (int j = 0; j < H; ++j) o |= ((h >> j) & 1u) << sw.high_bits[j];
                hoff[h] = o;
            }
            uint32_t outer_bits[32];
            int n_outer = 0;
            {
                uint32_t in_tile = lmask;
                for (int j = 0; j < H; ++j) in_tile |= 1u << sw.high_bits[j];
                for (int b = 0; b < a.n; ++b)
                    if (!((in_tile >> b) & 1u)) outer_bits[n_outer++] = b;
            }
            // the Paulis of the sweep's channels (state independent, the gate-by-gate kernel's counters)
            for (int c = tid; c < 2 * nops; c += nthr) {
                const int i = c >> 1, j = c & 1;
                int p = 0;
                if (a.p_dep > 0 && j < sops[i].k) {
                    const double u = Philox::uniform(uint32_t(sops[i].gate), uint32_t(t), 2u * j, a.seed0, a.seed1);
                    if (u >= 1.0 - a.p_dep) p = 1 + min(2, int((u - (1.0 - a.p_dep)) / (a.p_dep / 3.0)));
                }
                pk[i][j] = uint8_t(p);
            }
            if (tid == 0) s_njump = 0;
            __syncthreads();
            // each op's matrix with its Paulis folded into the rows (X swaps, Y swaps with -i / i, Z negates
            // the |1> row of its site); the first op of the sweep also carries the prescale 1 / sqrt(N_end)
            for (int i = tid; i < nops; i += nthr) {
                const TrajOpDesc& op = sops[i];
                const int D = 1 << op.k;
                C M[16];
                const T ps = i == 0 ? T(s_prescale) : T(1);
                for (int e = 0; e < D * D; ++e) {
                    const C x = mats[op.mat + e];
                    M[e] = mk<T>(x.x * ps, x.y * ps);
                }
                bool diag = (op.flags & 1) != 0;
                for (int j = 0; j < op.k; ++j) {
                    const int pj = pk[i][j];
                    if (pj == 0) continue;
                    if (pj != 3) diag = false;
                    const int bit = 1 << (op.k - 1 - j);
                    for (int r = 0; r < D; ++r) {
                        if (r & bit) continue;
                        for (int c = 0; c < D; ++c) {
                            const C lo = M[r * D + c], hi = M[(r | bit) * D + c];
                            if (pj == 1) {
                                M[r * D + c] = hi;
                                M[(r | bit) * D + c] = lo;
                            } else if (pj == 2) {
                                M[r * D + c] = mk<T>(hi.y, -hi.x);
                                M[(r | bit) * D + c] = mk<T>(-lo.y, lo.x);
                            } else {
                                M[(r | bit) * D + c] = mk<T>(-hi.x, -hi.y);
                            }
                        }
                    }
                }
                for (int e = 0; e < D * D; ++e) sm.msh[size_t(i) * 16 + e] = M[e];
                sm.dflag[i] = diag ? 1 : 0;
            }
            const uint64_t tiles = uint64_t(1) << (a.n - m);
            auto base_of = [&](uint64_t w) -> uint32_t {
                uint32_t b = 0;
                for (int j = 0; j < n_outer; ++j) b |= uint32_t((w >> j) & 1ull) << outer_bits[j];
                return b;
            };
            auto load = [&](uint64_t w, C* buf) {
                const uint32_t base = base_of(w);
                if (src) {
                    for (uint32_t e = per16 * tid; e < (1u << m); e += per16 * nthr)
                        traj_cp16(buf + tswz<T>(e), src + (base + hoff[e >> L] + (e & lmask)));
                } else {
                    for (uint32_t e = tid; e < (1u << m); e += nthr) {
                        const uint32_t gi = base + hoff[e >> L] + (e & lmask);
                        buf[tswz<T>(e)] = mk<T>(gi == 0 ? T(1) : T(0), T(0));
                    }
                }
                asm volatile("cp.async.commit_group;" ::: "memory");
            };
            for (int pass = 0; pass <= kTrajMaxJumps; ++pass) {
                // damping of every (op, site): K0, or the replayed jumps of this sweep
                for (int c = tid; c < 2 * nops; c += nthr) {
                    sm.dmode[c] = damp ? 1 : 0;
                    sm.djump[c] = T(0);
                }
                for (int c = tid; c < nwarps * 2 * nops; c += nthr)
                    wacc_zero(sm.chw_w[size_t(c / (2 * nops)) * (2 * kTrajMaxOps) + (c % (2 * nops))]);
                __syncthreads();
                if (tid == 0)
                    for (int q = 0; q < s_njump; ++q) {
                        sm.dmode[2 * jop[q] + jsite[q]] = 2;
                        sm.djump[2 * jop[q] + jsite[q]] = T(sqrt(a.gamma) * jscale[q]);
                    }
                __syncthreads();
                load(0, bufs);
                for (uint64_t w = 0; w < tiles; ++w) {
                    C* cur = bufs + (size_t(a.nbuf == 2 ? (w & 1) : 0) << m);
                    if (a.nbuf == 2 && w + 1 < tiles) {
                        load(w + 1, bufs + (size_t((w + 1) & 1) << m));
                        asm volatile("cp.async.wait_group 1;" ::: "memory");
                    } else {
                        asm volatile("cp.async.wait_group 0;" ::: "memory");
                    }
                    __syncthreads();
                    traj_tile_dispatch<T, traj_rmax<T>()>(cur, m, sops, nops, sm, damp, s0, tid, nthr);
                    const uint32_t base = base_of(w);
                    for (uint32_t e = per16 * tid; e < (1u << m); e += per16 * nthr)
                        *reinterpret_cast<float4*>(dst + (base + hoff[e >> L] + (e & lmask))) =
                            *reinterpret_cast<const float4*>(cur + tswz<T>(e));
                    __syncthreads();  // the buffer is free for the copy issued two tiles later
                    if (a.nbuf == 1 && w + 1 < tiles) load(w + 1, bufs);
                }
                // the weights, summed over the warps in a fixed order
                for (int c = tid; c < 2 * nops; c += nthr) {
                    double x = 0.0;
                    for (int wp = 0; wp < nwarps; ++wp) x += wacc_value(sm.chw_w[size_t(wp) * (2 * kTrajMaxOps) + c]);
                    chw[c] = x;
                }
                __syncthreads();
                // the sweep's channels in order: where does the no-jump norm fall below the threshold?
                if (tid == 0) {
                    s_replay = 0;
                    double N = 1.0;
                    if (damp) {
                        // channels up to the last jump recorded in this sweep are decided; after it the
                        // replay renormalised the state, so the walk restarts there with N = 1
                        int i0 = 0, j0 = 0;
                        if (s_njump > 0) {
                            i0 = jop[s_njump - 1];
                            j0 = jsite[s_njump - 1] + 1;
                        }
                        for (int i = i0; i < nops && !s_replay; ++i) {
                            const int k = sops[i].k;
                            for (int j = (i == i0 ? j0 : 0); j < k; ++j) {
                                const double Wc = chw[2 * i + j];
                                const double Nn = N - a.gamma * Wc;
                                if (Nn < s_r) {
                                    if (s_njump >= kTrajMaxJumps) {
                                        atomicExch(&g_traj_status, 1);  // too many jumps in one sweep: not replayed
                                        i = nops;
                                        break;
                                    }
                                    jop[s_njump] = i;
                                    jsite[s_njump] = j;
                                    jscale[s_njump] = 1.0 / sqrt(a.gamma * Wc);
                                    ++s_njump;
                                    const int idx = s_jumps_total++;
                                    if (idx < a.max_log && jump_log) {
                                        jump_log[(t * a.max_log + idx) * 2] = sops[i].gate;
                                        jump_log[(t * a.max_log + idx) * 2 + 1] = j;
                                    }
                                    s_r = Philox::uniform4(uint32_t(idx + 1), uint32_t(t), 0u, 2u, a.seed0, a.seed1);
                                    s_replay = 1;
                                    break;
                                }
                                N = Nn;
                            }
                        }
                    }
                    if (!s_replay) {
                        s_r = s_r / N;
                        s_prescale = 1.0 / sqrt(N);
                    }
                }
                __syncthreads();
                if (!s_replay) break;
            }
            src = dst;
            dst = (dst == own) ? scratch : own;
        }
        // the normalised state into the trajectory's slot
        {
            const T sc = T(s_prescale);
            if (src) {
                for (uint64_t e = tid; e < dim; e += nthr) {
                    const C v = src[e];
                    own[e] = mk<T>(v.x * sc, v.y * sc);
                }
            } else {
                for (uint64_t e = tid; e < dim; e += nthr) own[e] = mk<T>(e == 0 ? T(1) : T(0), T(0));
            }
        }
        if (tid == 0 && jump_count) jump_count[t] = s_jumps_total;
        __syncthreads();
    }
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

namespace {

template <typename T>
size_t traj_smem_bytes(int mmax, int hmax, int nbuf) {
    (void)hmax;
    return sizeof(cplx<T>) * (size_t(nbuf) << mmax) + traj_aux_bytes<T>();
}

template <typename T>
int traj_grid(int mmax, int hmax, int64_t ntraj, int* nbuf_out, size_t* smem_out) {
    auto kern = traj_run_kernel<T>;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess)
            return check_launch("trajectory kernel attribute");
        attr = true;
    }
    for (int nbuf = 2; nbuf >= 1; --nbuf) {
        const size_t smem = traj_smem_bytes<T>(mmax, hmax, nbuf);
        if (smem > 200 * 1024) continue;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTrajThreads, smem) != cudaSuccess)
            return check_launch("trajectory kernel occupancy");
        if (per_sm < 1) continue;
        int64_t grid = int64_t(per_sm) * sm_count();
        if (grid > ntraj) grid = ntraj;
        *nbuf_out = nbuf;
        *smem_out = smem;
        return int(grid);
    }
    return set_error(QGB_EINVAL, "trajectory tile of 2^%d amplitudes does not fit in shared memory", mmax);
}

int traj_check_tables(int n, const TrajSweepDesc* sweeps, int nsweeps, const TrajOpDesc* ops, int nops_total,
                      int64_t mat_elems, int* mmax, int* hmax, int dtype) {
    *mmax = 1;
    *hmax = 0;
    const int lmin = dtype == QGB_C64 ? 1 : 0;
    for (int s = 0; s < nsweeps; ++s) {
        const TrajSweepDesc& sw = sweeps[s];
        const int m = sw.L + sw.H;
        if (sw.L < lmin || sw.H < 0 || sw.H > QGB_SWEEP_MAX_HIGH || m > n || m > 14)
            return set_error(QGB_EINVAL, "sweep %d: tile geometry L=%d H=%d invalid for n=%d", s, sw.L, sw.H, n);
        int prev = sw.L - 1;
        for (int j = 0; j < sw.H; ++j) {
            if (sw.high_bits[j] <= prev || sw.high_bits[j] >= n)
                return set_error(QGB_EINVAL, "sweep %d: high bits must be ascending, >= L and < n", s);
            prev = sw.high_bits[j];
        }
        if (sw.op_begin < 0 || sw.op_end < sw.op_begin || sw.op_end > nops_total || sw.op_end - sw.op_begin > kTrajMaxOps ||
            sw.op_end == sw.op_begin)
            return set_error(QGB_EINVAL, "sweep %d: op range [%d, %d) invalid", s, sw.op_begin, sw.op_end);
        if (m > *mmax) *mmax = m;
        if (sw.H > *hmax) *hmax = sw.H;
        const int R = m < (dtype == QGB_C64 ? 4 : 3) ? m : (dtype == QGB_C64 ? 4 : 3);
        int run_left = 0;
        const int32_t* rpos = nullptr;
        for (int i = sw.op_begin; i < sw.op_end; ++i) {
            const TrajOpDesc& op = ops[i];
            if (run_left == 0) {
                if (op.run < 1 || i + op.run > sw.op_end)
                    return set_error(QGB_EINVAL, "op %d: run length %d invalid in its sweep", i, op.run);
                uint32_t seen = 0;
                for (int j = 0; j < R; ++j) {
                    const int p = op.run_pos[j];
                    if (p < 0 || p >= m || ((seen >> p) & 1u)) return set_error(QGB_EINVAL, "op %d: run positions invalid", i);
                    seen |= 1u << p;
                }
                run_left = op.run;
                rpos = op.run_pos;
            } else if (op.run != 0) {
                return set_error(QGB_EINVAL, "op %d opens a run inside another run", i);
            }
            --run_left;
            if (op.k < 1 || op.k > 2 || op.k > m) return set_error(QGB_EINVAL, "op %d: width %d invalid", i, op.k);
            for (int j = 0; j < op.k; ++j) {
                if (op.pos[j] < 0 || op.pos[j] >= m) return set_error(QGB_EINVAL, "op %d: tile position out of range", i);
                if (op.lpos[j] < 0 || op.lpos[j] >= R || rpos[op.lpos[j]] != op.pos[j])
                    return set_error(QGB_EINVAL, "op %d: local position does not match its run", i);
            }
            if (op.k == 2 && op.pos[0] == op.pos[1]) return set_error(QGB_EINVAL, "op %d: repeated tile position", i);
            if (op.gate < 0 || op.mat < 0 || op.mat + (int64_t(1) << (2 * op.k)) > mat_elems)
                return set_error(QGB_EINVAL, "op %d: gate index or matrix offset out of range", i);
        }
    }
    return QGB_OK;
}

}  // namespace

extern "C" size_t qgb_traj_sweep_bytes(void) { return sizeof(TrajSweepDesc); }
extern "C" size_t qgb_traj_op_bytes(void) { return sizeof(TrajOpDesc); }

extern "C" size_t qgb_traj_run_scratch_bytes(int dtype, int n, int tile_bits, int64_t ntraj) {
    if ((dtype != QGB_C64 && dtype != QGB_C128) || n < 1 || n > 30 || tile_bits < 1 || tile_bits > 14 || ntraj < 1)
        return 0;
    const int m = tile_bits < n ? tile_bits : n;
    int nbuf = 0;
    size_t smem = 0;
    const int grid = dtype == QGB_C64 ? traj_grid<float>(m, QGB_SWEEP_MAX_HIGH, ntraj, &nbuf, &smem)
                                      : traj_grid<double>(m, QGB_SWEEP_MAX_HIGH, ntraj, &nbuf, &smem);
    if (grid <= 0) return 0;
    const size_t isz = dtype == QGB_C64 ? 8 : 16;
    return 256 + size_t(grid) * (size_t(1) << n) * isz;
}

extern "C" int qgb_traj_run(void* sv, int dtype, int n, int64_t ntraj, int64_t stride, const qgb_traj_sweep* sweeps_host,
                            const qgb_traj_sweep* sweeps_dev, int nsweeps, const qgb_traj_op* ops_host,
                            const qgb_traj_op* ops_dev, int nops, const void* mats, int64_t mat_elems, double p_dep, double gamma, uint64_t seed, int* jump_count,
                            int* jump_log, int max_log, void* scratch, size_t scratch_bytes, void* stream) {
    if (!sv || !sweeps_host || !sweeps_dev || !ops_host || !ops_dev || !mats || !scratch)
        return set_error(QGB_EINVAL, "null pointer");
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    if (n < 1 || n > 30) return set_error(QGB_EINVAL, "n=%d invalid (trajectories of 1 to 30 qubits)", n);
    if (ntraj < 1 || ntraj > (int64_t(1) << 30)) return set_error(QGB_EINVAL, "ntraj %lld out of range", (long long)ntraj);
    if (ntraj > 1 && stride < (int64_t(1) << n)) return set_error(QGB_EINVAL, "trajectory stride too small");
    if (nsweeps < 0 || nops < 0) return set_error(QGB_EINVAL, "negative table size");
    if (p_dep < 0 || p_dep > 1 || gamma < 0 || gamma >= 1) return set_error(QGB_EINVAL, "noise parameters out of range");
    if (max_log < 0 || (max_log > 0 && !jump_log)) return set_error(QGB_EINVAL, "jump log missing");
    const size_t isz = dtype == QGB_C64 ? 8 : 16;
    if ((reinterpret_cast<uintptr_t>(sv) & 15) || (ntraj > 1 && (stride * int64_t(isz)) % 16) ||
        (reinterpret_cast<uintptr_t>(scratch) & 15))
        return set_error(QGB_EINVAL, "state, stride and scratch must be 16-byte aligned");
    if (reinterpret_cast<uintptr_t>(mats) % isz) return set_error(QGB_EINVAL, "matrix buffer misaligned");
    int mmax = 1, hmax = 0;
    int rc = traj_check_tables(n, reinterpret_cast<const TrajSweepDesc*>(sweeps_host), nsweeps,
                               reinterpret_cast<const TrajOpDesc*>(ops_host), nops, mat_elems, &mmax, &hmax, dtype);
    if (rc) return rc;
    int nbuf = 0;
    size_t smem = 0;
    // shared memory sized for the largest high-bit table, as qgb_traj_run_scratch_bytes assumes
    (void)hmax;
    const int grid = dtype == QGB_C64 ? traj_grid<float>(mmax, QGB_SWEEP_MAX_HIGH, ntraj, &nbuf, &smem)
                                      : traj_grid<double>(mmax, QGB_SWEEP_MAX_HIGH, ntraj, &nbuf, &smem);
    if (grid <= 0) return grid < 0 ? grid : set_error(QGB_ECUDA, "no trajectory CTA fits on an SM");
    const size_t need = 256 + size_t(grid) * (size_t(1) << n) * isz;
    if (scratch_bytes < need) return set_error(QGB_ESCRATCH, "trajectory scratch of %zu bytes needed", need);
    cudaStream_t st = (cudaStream_t)stream;
    int* queue = static_cast<int*>(scratch);
    if (cudaMemsetAsync(queue, 0, sizeof(int), st) != cudaSuccess) return check_launch("trajectory queue reset");
    void* ping = static_cast<unsigned char*>(scratch) + 256;
    TrajRunArgs a{};
    a.n = n;
    a.ntraj = ntraj;
    a.stride = ntraj > 1 ? stride : 0;
    a.nsweeps = nsweeps;
    a.p_dep = p_dep;
    a.gamma = gamma;
    a.seed0 = uint32_t(seed);
    a.seed1 = uint32_t(seed >> 32);
    a.nbuf = nbuf;
    a.mmax = mmax;
    a.max_log = max_log;
    const TrajSweepDesc* sd = reinterpret_cast<const TrajSweepDesc*>(sweeps_dev);
    const TrajOpDesc* od = reinterpret_cast<const TrajOpDesc*>(ops_dev);
    if (dtype == QGB_C64)
        traj_run_kernel<float><<<grid, kTrajThreads, smem, st>>>((float2*)sv, (float2*)ping, sd, od,
                                                                  (const float2*)mats, queue, jump_count, jump_log, a);
    else
        traj_run_kernel<double><<<grid, kTrajThreads, smem, st>>>((double2*)sv, (double2*)ping, sd, od,
                                                                   (const double2*)mats, queue, jump_count, jump_log, a);
    return check_launch("trajectory kernel");
}

namespace qgb_host {
int traj_status_read_clear() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, qgb::g_traj_status, sizeof(int)) != cudaSuccess) return -1;
    if (v != 0) {
        const int z = 0;
        cudaMemcpyToSymbol(qgb::g_traj_status, &z, sizeof(int));
    }
    return v;
}
}  // namespace qgb_host
