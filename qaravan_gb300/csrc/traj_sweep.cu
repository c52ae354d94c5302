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
constexpr int kTrajThreads = 256;

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

// Amplitude damping of the site at matrix bit `bit` of a group of D amplitudes
// in registers: W += weight of the |1> components; then K0 (mode 1) or the
// jump sc * K1 (mode 2).
template <int D, typename C, typename T>
__device__ __forceinline__ void traj_damp(C (&v)[D], int bit, int mode, T s0, T sj, float& w) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
        if (!(c & bit)) continue;
        w += float(v[c].x) * float(v[c].x) + float(v[c].y) * float(v[c].y);
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

// One op (gate with the sampled Paulis folded into its rows, then amplitude
// damping of each site) on every group of a staged tile.
template <typename T, int K>
__device__ __forceinline__ void traj_tile_op(cplx<T>* __restrict__ tile, int m, const TrajOpDesc& op,
                                             const cplx<T>* __restrict__ mat, T prescale, const uint8_t* pk,
                                             const int* dmode, const T* djump, T s0, double* chw, int tid,
                                             int nthr) {
    using C = cplx<T>;
    constexpr int D = 1 << K;
    C M[D * D];
#pragma unroll
    for (int i = 0; i < D * D; ++i) {
        const C e = __ldg(&mat[i]);
        M[i] = mk<T>(e.x * prescale, e.y * prescale);
    }
    // Paulis after the gate: rows r and r ^ bit of site j (X swaps, Y swaps with -i / i, Z negates the |1> row)
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const int p = pk[j];
        if (p == 0) continue;
        const int bit = 1 << (K - 1 - j);
#pragma unroll
        for (int r = 0; r < D; ++r) {
            if (r & bit) continue;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const C lo = M[r * D + c], hi = M[(r | bit) * D + c];
                if (p == 1) {
                    M[r * D + c] = hi;
                    M[(r | bit) * D + c] = lo;
                } else if (p == 2) {
                    M[r * D + c] = mk<T>(hi.y, -hi.x);
                    M[(r | bit) * D + c] = mk<T>(-lo.y, lo.x);
                } else {
                    M[(r | bit) * D + c] = mk<T>(-hi.x, -hi.y);
                }
            }
        }
    }
    int pos[K], srt[K];
#pragma unroll
    for (int j = 0; j < K; ++j) pos[j] = srt[j] = op.pos[j];
    if (K == 2 && srt[0] > srt[1]) {
        const int x = srt[0];
        srt[0] = srt[1];
        srt[1] = x;
    }
    uint32_t soff[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
        uint32_t o = 0;
#pragma unroll
        for (int j = 0; j < K; ++j) o |= uint32_t((c >> (K - 1 - j)) & 1) << pos[j];
        soff[c] = tswz<T>(o);
    }
    float w[K];
#pragma unroll
    for (int j = 0; j < K; ++j) w[j] = 0.f;
    const uint32_t groups = 1u << (m - K);
    for (uint32_t g = tid; g < groups; g += nthr) {
        uint32_t base = g;
#pragma unroll
        for (int j = 0; j < K; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((1u << srt[j]) - 1));
        const uint32_t sb = tswz<T>(base);
        C v[D], o[D];
#pragma unroll
        for (int c = 0; c < D; ++c) v[c] = tile[sb ^ soff[c]];
#pragma unroll
        for (int r = 0; r < D; ++r) {
            C acc = mk<T>(0, 0);
#pragma unroll
            for (int c = 0; c < D; ++c) cfma(acc, M[r * D + c], v[c]);
            o[r] = acc;
        }
#pragma unroll
        for (int j = 0; j < K; ++j)
            if (dmode[j]) traj_damp<D>(o, 1 << (K - 1 - j), dmode[j], s0, djump[j], w[j]);
#pragma unroll
        for (int c = 0; c < D; ++c) tile[sb ^ soff[c]] = o[c];
    }
    if (chw) {
        // the sites' weights: warp sums, one shared-memory atomic per warp and site
#pragma unroll
        for (int j = 0; j < K; ++j) {
            float x = w[j];
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) x += __shfl_down_sync(0xffffffffu, x, s);
            if ((tid & 31) == 0 && dmode[j]) atomicAdd(&chw[j], double(x));
        }
    }
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
    __shared__ double chw[2 * kTrajMaxOps];        // per (op, site) of the sweep: weight of |1> before damping
    __shared__ uint8_t pk[kTrajMaxOps][2];          // sampled Paulis
    __shared__ int jop[kTrajMaxJumps], jsite[kTrajMaxJumps];
    __shared__ double jscale[kTrajMaxJumps];
    __shared__ int s_traj, s_njump, s_replay;
    __shared__ double s_r, s_prescale;
    __shared__ int s_jumps_total;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const uint64_t dim = uint64_t(1) << a.n;
    C* scratch = pingpong + uint64_t(blockIdx.x) * dim;
    const T s0 = T(sqrt(1.0 - a.gamma));
    const T sqg = T(sqrt(a.gamma));
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
                const TrajOpDesc& op = ops[sw.op_begin + i];
                int p = 0;
                if (a.p_dep > 0 && j < op.k) {
                    const double u = Philox::uniform(uint32_t(op.gate), uint32_t(t), 2u * j, a.seed0, a.seed1);
                    if (u >= 1.0 - a.p_dep) p = 1 + min(2, int((u - (1.0 - a.p_dep)) / (a.p_dep / 3.0)));
                }
                pk[i][j] = uint8_t(p);
            }
            if (tid == 0) s_njump = 0;
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
                for (int c = tid; c < 2 * nops; c += nthr) chw[c] = 0.0;
                __syncthreads();
                const T pre = T(s_prescale);
                const int njump = s_njump;
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
                    int jn = 0;  // next recorded jump of this pass
                    for (int i = 0; i < nops; ++i) {
                        const TrajOpDesc op = ops[sw.op_begin + i];
                        int dm[2] = {a.gamma > 0 ? 1 : 0, a.gamma > 0 ? 1 : 0};
                        T dj[2] = {T(0), T(0)};
                        while (jn < njump && jop[jn] == i) {
                            dm[jsite[jn]] = 2;
                            dj[jsite[jn]] = T(double(sqg) * jscale[jn]);
                            ++jn;
                        }
                        const T ps = i == 0 ? pre : T(1);
                        double* cw = a.gamma > 0 ? &chw[2 * i] : nullptr;
                        if (op.k == 1)
                            traj_tile_op<T, 1>(cur, m, op, mats + op.mat, ps, pk[i], dm, dj, s0, cw, tid, nthr);
                        else
                            traj_tile_op<T, 2>(cur, m, op, mats + op.mat, ps, pk[i], dm, dj, s0, cw, tid, nthr);
                        __syncthreads();
                    }
                    const uint32_t base = base_of(w);
                    for (uint32_t e = per16 * tid; e < (1u << m); e += per16 * nthr)
                        *reinterpret_cast<float4*>(dst + (base + hoff[e >> L] + (e & lmask))) =
                            *reinterpret_cast<const float4*>(cur + tswz<T>(e));
                    __syncthreads();  // the buffer is free for the copy issued two tiles later
                    if (a.nbuf == 1 && w + 1 < tiles) load(w + 1, bufs);
                }
                // the sweep's channels in order: where does the no-jump norm fall below the threshold?
                if (tid == 0) {
                    s_replay = 0;
                    double N = 1.0;
                    if (a.gamma > 0) {
                        // channels up to the last jump recorded in this sweep are decided; after it the
                        // replay renormalised the state, so the walk restarts there with N = 1
                        int i0 = 0, j0 = 0;
                        if (s_njump > 0) {
                            i0 = jop[s_njump - 1];
                            j0 = jsite[s_njump - 1] + 1;
                        }
                        for (int i = i0; i < nops && !s_replay; ++i) {
                            const int k = ops[sw.op_begin + i].k;
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
                                        jump_log[(t * a.max_log + idx) * 2] = ops[sw.op_begin + i].gate;
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
            const C* from = src ? src : nullptr;
            if (from) {
                for (uint64_t e = tid; e < dim; e += nthr) {
                    const C v = from[e];
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
    return sizeof(cplx<T>) * (size_t(nbuf) << mmax) + sizeof(uint32_t) * (size_t(1) << hmax);
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
        for (int i = sw.op_begin; i < sw.op_end; ++i) {
            const TrajOpDesc& op = ops[i];
            if (op.k < 1 || op.k > 2 || op.k > m) return set_error(QGB_EINVAL, "op %d: width %d invalid", i, op.k);
            for (int j = 0; j < op.k; ++j)
                if (op.pos[j] < 0 || op.pos[j] >= m) return set_error(QGB_EINVAL, "op %d: tile position out of range", i);
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
