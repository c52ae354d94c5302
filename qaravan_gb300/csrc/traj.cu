// Batched noisy trajectories (Monte-Carlo wavefunction unravelling).
//
// The reference samples noisy circuits one at a time on the CPU
// (MonteCarloSim, tensorQ/monte_carlo_sim.py:14-35) and only for Pauli
// channels; amplitude damping exists only as a density-matrix superoperator
// (core/noise.py:29-49). Here all trajectories advance together, one gate at a
// time, each keeping its own normalised 2^n state:
//
//  * traj_gate_kernel: per (trajectory, block) CTA, apply the trajectory's op
//    on the union U of the gate's sites and the previous gate's sites (at
//    most 4 bits) to every group of 2^|U| amplitudes, in factors held in
//    registers: the previous gate's pending Kraus operators (normalised), then
//    the gate with the depolarising Paulis sampled for this trajectory and
//    gate folded in; accumulate |out|^2 per value of the gate sites' bits
//    (float64 partials).
//  * traj_decide_kernel: one thread per trajectory sums the partials into the
//    joint populations of the gate's sites and draws the amplitude-damping
//    branches site by site (exact sequential probabilities gamma * P(1)),
//    writing the normalised Kraus operators K0/sqrt(1-p) or K1/sqrt(p) that
//    the next traj_gate launch applies, and logging the branches.
//
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11), counter = (event, trajectory, stream,
// 0), key = the run's seed; 53-bit uniforms from two output words.
#include "philox.cuh"
#include "qgb_common.cuh"

namespace qgb {

struct TrajGateArgs {
    int n;
    int64_t ntraj, stride;
    int ku;            // |U|: union bits (0..4)
    int ubits[4];      // flat bits of U, matrix order (bit ku-1-j of the local index <-> ubits[j])
    int kg;            // gate width (0..2); gate site j is U position gpos[j]
    int gpos[2];
    int kp;            // pending Kraus sites (0..2); site j is U position ppos[j]
    int ppos[2];
    double p_dep;      // depolarising probability per gate site (0 = none)
    uint32_t seed0, seed1, event;
    int nblk;
    int log_paulis;    // write the sampled Pauli indices to the log
    // staged access (a union bit below 5): a warp's 32 groups span the union bits and
    // the 5 lowest other bits W (K + 5 bits, W's lowest five are bits 0..4); rank r of
    // W has global offset wg[r] and shared-memory offset ws[r] in the warp's
    // [component c][lane] array (row pitch 33)
    int staged;
    uint32_t wg[9], ws[9];
};

// v <- K on local position P (bit K_-1-P of the local index), K real 2x2.
template <int K_, int P, typename C, typename T>
__device__ __forceinline__ void kraus_at(C (&v)[1 << K_], T k00, T k01, T k10, T k11) {
    constexpr int D = 1 << K_, bit = 1 << (K_ - 1 - P);
#pragma unroll
    for (int c = 0; c < D; ++c) {
        if (c & bit) continue;
        const C a = v[c], b = v[c | bit];
        v[c].x = k00 * a.x + k01 * b.x;
        v[c].y = k00 * a.y + k01 * b.y;
        v[c | bit].x = k10 * a.x + k11 * b.x;
        v[c | bit].y = k10 * a.y + k11 * b.y;
    }
}

template <int K_, typename C, typename T>
__device__ __forceinline__ void kraus_dispatch(C (&v)[1 << K_], int p, const T k[4]) {
    switch (p) {
        case 0: kraus_at<K_, 0>(v, k[0], k[1], k[2], k[3]); break;
        case 1: if constexpr (K_ > 1) kraus_at<K_, 1>(v, k[0], k[1], k[2], k[3]); break;
        case 2: if constexpr (K_ > 2) kraus_at<K_, 2>(v, k[0], k[1], k[2], k[3]); break;
        case 3: if constexpr (K_ > 3) kraus_at<K_, 3>(v, k[0], k[1], k[2], k[3]); break;
    }
}

// The trajectory's op on the union U of the gate's sites (local positions
// 0..KG-1, the top bits of the local index) and the pending sites, applied in
// factors: out = (Paulis . G on the gate positions) (K_1 K_0 on the pending
// positions) v. The Kraus operators of amplitude damping are real (diag(1,
// sqrt(1-gamma)) / sqrt(1-p) or sqrt(gamma/p) |0><1|); the Paulis, sampled
// per trajectory, are folded into the gd x gd gate matrix in registers.
// Per amplitude that is 4 * (kp + gd) real FMAs instead of the 4 * 2^K of the
// composed 2^K x 2^K product.
template <typename T, int K, int KG, bool STAGED>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? (K <= 2 ? 4 : 2) : 1) traj_gate_kernel(cplx<T>* __restrict__ sv, const cplx<T>* __restrict__ gate,
                                                        const cplx<T>* __restrict__ kraus, double* __restrict__ partials,
                                                        uint8_t* __restrict__ pauli_log, const __grid_constant__ TrajGateArgs a) {
    using C = cplx<T>;
    constexpr int D = 1 << K, GD = 1 << KG, LOW = K - KG;
    __shared__ double red[8][4];
    __shared__ C stg[STAGED ? 8 : 1][STAGED ? D * 33 : 1];
    const int64_t t = blockIdx.y;
    // ---- G' = (P_0 x P_1) G on the gate positions, every thread the same values
    C G[GD * GD];
#pragma unroll
    for (int e = 0; e < GD * GD; ++e) G[e] = KG > 0 ? gate[e] : mk<T>(T(1), T(0));
    if constexpr (KG > 0) {
        if (a.p_dep > 0) {
#pragma unroll
            for (int j = 0; j < KG; ++j) {
                const double u = Philox::uniform(a.event, uint32_t(t), 2u * j, a.seed0, a.seed1);
                // I with 1-p, X, Y, Z with p/3 each
                int pk = 0;
                if (u >= 1.0 - a.p_dep) pk = 1 + min(2, int((u - (1.0 - a.p_dep)) / (a.p_dep / 3.0)));
                if (a.log_paulis && blockIdx.x == 0 && threadIdx.x == 0) pauli_log[t * 2 + j] = uint8_t(pk);
                if (pk == 0) continue;
                const int bit = 1 << (KG - 1 - j);
                // rows r (bit clear) and r | bit: X swaps them, Y swaps with (-i, i), Z negates the second
#pragma unroll
                for (int r = 0; r < GD; ++r) {
                    if (r & bit) continue;
#pragma unroll
                    for (int c = 0; c < GD; ++c) {
                        const C lo = G[r * GD + c], hi = G[(r | bit) * GD + c];
                        if (pk == 1) {
                            G[r * GD + c] = hi;
                            G[(r | bit) * GD + c] = lo;
                        } else if (pk == 2) {
                            G[r * GD + c] = mk<T>(hi.y, -hi.x);        // -i * hi
                            G[(r | bit) * GD + c] = mk<T>(-lo.y, lo.x);  //  i * lo
                        } else {
                            G[(r | bit) * GD + c] = mk<T>(-hi.x, -hi.y);
                        }
                    }
                }
            }
        }
    }
    T kr[2][4];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
#pragma unroll
        for (int e = 0; e < 4; ++e) kr[j][e] = j < a.kp ? kraus[(t * 2 + j) * 4 + e].x : T(0);
    }
    int srt[K];
#pragma unroll
    for (int j = 0; j < K; ++j) srt[j] = a.ubits[j];
#pragma unroll
    for (int i = 1; i < K; ++i)
#pragma unroll
        for (int j = i; j > 0; --j)
            if (srt[j - 1] > srt[j]) {
                const int x = srt[j];
                srt[j] = srt[j - 1];
                srt[j - 1] = x;
            }
    uint32_t m[K];  // n <= 32: offsets within a trajectory's state fit 32 bits
#pragma unroll
    for (int j = 0; j < K; ++j) m[j] = uint32_t(1) << a.ubits[j];
    C* s = sv + t * a.stride;
    const uint64_t groups = uint64_t(1) << (a.n - K), step = uint64_t(a.nblk) * blockDim.x;
    // per-thread partial sums in the state's precision (a few dozen terms each; float64 across threads)
    T pop[GD];
#pragma unroll
    for (int b = 0; b < GD; ++b) pop[b] = 0;
    uint32_t ws_lane = 0;  // staged: this lane's contribution to the shared-memory offset
    if constexpr (STAGED) {
#pragma unroll
        for (int r = 0; r < 5; ++r)
            if ((threadIdx.x >> r) & 1) ws_lane += a.ws[r];
    }
    for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < groups; g += step) {
        uint64_t base = g;
        if constexpr (STAGED) base &= ~uint64_t(31);
#pragma unroll
        for (int j = 0; j < K; ++j) base = ((base >> srt[j]) << (srt[j] + 1)) | (base & ((uint64_t(1) << srt[j]) - 1));
        C* sb = s + base;
        C v[D];
        if constexpr (STAGED) {
            // the warp's 32 x D amplitudes in memory order, 256 contiguous bytes per load
            const int lane = threadIdx.x & 31;
            C* st = stg[threadIdx.x >> 5];
#pragma unroll
            for (int i = 0; i < D; ++i) {
                uint32_t go = lane, so = ws_lane;
#pragma unroll
                for (int b = 0; b < K; ++b)
                    if ((i >> b) & 1) {
                        go += a.wg[5 + b];
                        so += a.ws[5 + b];
                    }
                st[so] = sb[go];
            }
            __syncwarp();
#pragma unroll
            for (int c = 0; c < D; ++c) v[c] = st[c * 33 + lane];
        } else {
#pragma unroll
            for (int c = 0; c < D; ++c) {
                uint32_t o = 0;
#pragma unroll
                for (int j = 0; j < K; ++j)
                    if ((c >> (K - 1 - j)) & 1) o += m[j];
                v[c] = sb[o];
            }
        }
        if (a.kp > 0) kraus_dispatch<K>(v, a.ppos[0], kr[0]);
        if (a.kp > 1) kraus_dispatch<K>(v, a.ppos[1], kr[1]);
        if constexpr (KG > 0) {
#pragma unroll
            for (int l = 0; l < (1 << LOW); ++l) {
                C in[GD];
#pragma unroll
                for (int c = 0; c < GD; ++c) in[c] = v[(c << LOW) | l];
#pragma unroll
                for (int r = 0; r < GD; ++r) {
                    C acc = mk<T>(0, 0);
#pragma unroll
                    for (int c = 0; c < GD; ++c) cfma(acc, G[r * GD + c], in[c]);
                    v[(r << LOW) | l] = acc;
                    pop[r] += acc.x * acc.x + acc.y * acc.y;
                }
            }
        }
        if constexpr (STAGED) {
            const int lane = threadIdx.x & 31;
            C* st = stg[threadIdx.x >> 5];
#pragma unroll
            for (int c = 0; c < D; ++c) st[c * 33 + lane] = v[c];
            __syncwarp();
#pragma unroll
            for (int i = 0; i < D; ++i) {
                uint32_t go = lane, so = ws_lane;
#pragma unroll
                for (int b = 0; b < K; ++b)
                    if ((i >> b) & 1) {
                        go += a.wg[5 + b];
                        so += a.ws[5 + b];
                    }
                sb[go] = st[so];
            }
            __syncwarp();  // every lane's reads done before the next groups are staged
        } else {
#pragma unroll
            for (int c = 0; c < D; ++c) {
                uint32_t o = 0;
#pragma unroll
                for (int j = 0; j < K; ++j)
                    if ((c >> (K - 1 - j)) & 1) o += m[j];
                sb[o] = v[c];
            }
        }
    }
    // block reduction of the joint populations of the gate sites -> partials[(t * nblk + blk) * 4 + b]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        double x = b < GD && KG > 0 ? double(pop[b < GD ? b : 0]) : 0.0;
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][b] = x;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double x = 0;
        for (int w = 0; w < int(blockDim.x / 32); ++w) x += red[w][threadIdx.x];
        partials[(t * a.nblk + blockIdx.x) * 4 + threadIdx.x] = x;
    }
}

struct TrajDecideArgs {
    int64_t ntraj;
    int ku, nblk;
    int kg, gpos[2];   // gate sites as U positions (the damped sites, in order)
    double gamma;
    uint32_t seed0, seed1, event;
};

// One thread per trajectory: joint populations of the gate sites -> sequential
// amplitude-damping branches -> normalised Kraus operators for the next launch.
template <typename T>
__global__ void traj_decide_kernel(const double* __restrict__ partials, cplx<T>* __restrict__ kraus,
                                   uint8_t* __restrict__ jump_log, const __grid_constant__ TrajDecideArgs a) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= a.ntraj) return;
    double P[4] = {0, 0, 0, 0};  // P[2*b0 + b1] (kg = 2) or P[b0] (kg = 1) over the gate sites' bits
    for (int blk = 0; blk < a.nblk; ++blk) {
        const double* p = partials + (t * a.nblk + blk) * 4;
        for (int b = 0; b < 4; ++b) P[b] += p[b];
    }
    const double g = a.gamma;
    for (int j = 0; j < a.kg; ++j) {
        // population of site j being 1
        double tot = 0, p1 = 0;
        for (int i = 0; i < (1 << a.kg); ++i) {
            tot += P[i];
            if ((i >> (a.kg - 1 - j)) & 1) p1 += P[i];
        }
        const double pj = tot > 0 ? g * p1 / tot : 0.0;
        const double u = Philox::uniform(a.event, uint32_t(t), 2u * j + 1u, a.seed0, a.seed1);
        const bool jump = u < pj;
        cplx<T>* K = kraus + (t * 2 + j) * 4;
        if (jump) {
            // K1 = sqrt(g) |0><1| / sqrt(pj)
            K[0] = mk<T>(0, 0);
            K[1] = mk<T>(T(sqrt(g / pj)), 0);
            K[2] = mk<T>(0, 0);
            K[3] = mk<T>(0, 0);
            // K1 annihilates the site-0 components and moves site-1 weight (times g) to site 0
            for (int i = 0; i < (1 << a.kg); ++i)
                if ((i >> (a.kg - 1 - j)) & 1) {
                    P[i & ~(1 << (a.kg - 1 - j))] = g * P[i];
                    P[i] = 0;
                }
        } else {
            // K0 = diag(1, sqrt(1-g)) / sqrt(1-pj)
            const double s = 1.0 / sqrt(1.0 - pj);
            K[0] = mk<T>(T(s), 0);
            K[1] = mk<T>(0, 0);
            K[2] = mk<T>(0, 0);
            K[3] = mk<T>(T(s * sqrt(1.0 - g)), 0);
            for (int i = 0; i < (1 << a.kg); ++i)
                if ((i >> (a.kg - 1 - j)) & 1) P[i] *= (1.0 - g);
        }
        if (jump_log) jump_log[t * 2 + j] = jump ? 1 : 0;
    }
}

}  // namespace qgb

using namespace qgb;
using namespace qgb_host;

namespace {

template <typename T, int K, int KG>
int launch_gate(void* sv, const void* gate, const void* kraus, double* partials, uint8_t* plog, const TrajGateArgs& a,
                cudaStream_t st) {
    dim3 grid(unsigned(a.nblk), unsigned(a.ntraj));
    if constexpr (sizeof(T) == 4) {
        if (a.staged) {
            traj_gate_kernel<T, K, KG, true><<<grid, 256, 0, st>>>((cplx<T>*)sv, (const cplx<T>*)gate,
                                                                   (const cplx<T>*)kraus, partials, plog, a);
            return check_launch("trajectory gate kernel");
        }
    }
    traj_gate_kernel<T, K, KG, false><<<grid, 256, 0, st>>>((cplx<T>*)sv, (const cplx<T>*)gate, (const cplx<T>*)kraus,
                                                            partials, plog, a);
    return check_launch("trajectory gate kernel");
}

template <typename T, int K>
int launch_gate(void* sv, const void* gate, const void* kraus, double* partials, uint8_t* plog, const TrajGateArgs& a,
                cudaStream_t st) {
    switch (a.kg) {
        case 0: return launch_gate<T, K, 0>(sv, gate, kraus, partials, plog, a, st);
        case 1: return launch_gate<T, K, 1>(sv, gate, kraus, partials, plog, a, st);
        case 2: if constexpr (K >= 2) return launch_gate<T, K, 2>(sv, gate, kraus, partials, plog, a, st); break;
    }
    return set_error(QGB_EINVAL, "gate width %d with %d union bits", a.kg, a.ku);
}

template <typename T>
int dispatch_gate(void* sv, const void* gate, const void* kraus, double* partials, uint8_t* plog, const TrajGateArgs& a,
                  cudaStream_t st) {
    switch (a.ku) {
        case 1: return launch_gate<T, 1>(sv, gate, kraus, partials, plog, a, st);
        case 2: return launch_gate<T, 2>(sv, gate, kraus, partials, plog, a, st);
        case 3: return launch_gate<T, 3>(sv, gate, kraus, partials, plog, a, st);
        case 4: return launch_gate<T, 4>(sv, gate, kraus, partials, plog, a, st);
    }
    return set_error(QGB_EINVAL, "union of gate and pending sites has %d bits (1..4 supported)", a.ku);
}

}  // namespace

extern "C" int qgb_traj_blocks(int n) {
    // blocks per trajectory: about 16 groups per thread, at most 64 blocks
    const int64_t groups = int64_t(1) << (n > 4 ? n - 4 : 0);
    int64_t b = groups / (256 * 16);
    if (b < 1) b = 1;
    if (b > 64) b = 64;
    return int(b);
}

extern "C" int qgb_traj_step(void* sv, int dtype, int n, int64_t ntraj, int64_t stride, const int* sites, int k,
                             const void* gate, const int* prev_sites, int kprev, void* kraus, double p_dep,
                             double gamma, uint64_t seed, uint32_t event, double* partials, uint8_t* pauli_log,
                             uint8_t* jump_log, void* stream) {
    if (!sv || !kraus || !partials) return set_error(QGB_EINVAL, "null pointer");
    if (dtype != QGB_C64 && dtype != QGB_C128) return set_error(QGB_EINVAL, "dtype %d unknown", dtype);
    if (n < 1 || n > 32) return set_error(QGB_EINVAL, "n=%d invalid (trajectories of 1 to 32 qubits)", n);
    if (ntraj < 1 || ntraj > 65535) return set_error(QGB_EINVAL, "ntraj %lld not in [1, 65535]", (long long)ntraj);
    if (ntraj > 1 && stride < (int64_t(1) << n)) return set_error(QGB_EINVAL, "trajectory stride too small");
    if (k < 0 || k > 2 || kprev < 0 || kprev > 2) return set_error(QGB_EINVAL, "gate and pending widths must be 0..2");
    if (k > 0 && (!sites || !gate)) return set_error(QGB_EINVAL, "gate sites/matrix missing");
    if (kprev > 0 && !prev_sites) return set_error(QGB_EINVAL, "pending sites missing");
    if (p_dep < 0 || p_dep > 1 || gamma < 0 || gamma >= 1) return set_error(QGB_EINVAL, "noise parameters out of range");
    TrajGateArgs a{};
    a.n = n;
    a.ntraj = ntraj;
    a.stride = ntraj > 1 ? stride : 0;
    // union U: gate sites first, then pending sites not already present
    int ub[4], nu = 0;
    auto add = [&](int site) -> int {
        if (site < 0 || site >= n) return -1;
        const int bit = n - 1 - site;
        for (int i = 0; i < nu; ++i)
            if (ub[i] == bit) return i;
        ub[nu] = bit;
        return nu++;
    };
    a.kg = k;
    for (int j = 0; j < k; ++j) {
        const int p = add(sites[j]);
        if (p < 0) return set_error(QGB_EINVAL, "gate site out of range");
        for (int i = 0; i < j; ++i)
            if (a.gpos[i] == p) return set_error(QGB_EINVAL, "repeated gate site");
        a.gpos[j] = p;
    }
    a.kp = kprev;
    for (int j = 0; j < kprev; ++j) {
        const int p = add(prev_sites[j]);
        if (p < 0) return set_error(QGB_EINVAL, "pending site out of range");
        a.ppos[j] = p;
    }
    if (nu == 0) return QGB_OK;
    a.ku = nu;
    for (int j = 0; j < nu; ++j) a.ubits[j] = ub[j];
    // staged access when a union bit is below 5 (complex64, at least one warp of groups)
    int lowest = n;
    for (int j = 0; j < nu; ++j) lowest = ub[j] < lowest ? ub[j] : lowest;
    a.staged = (dtype == QGB_C64 && lowest < 5 && n - nu >= 5) ? 1 : 0;
    if (a.staged) {
        // W: the union bits and the 5 lowest other bits, ascending
        int lane_bits[5], nl = 0, w = 0;
        for (int b = 0; b < n && nl < 5; ++b) {
            bool in_u = false;
            for (int j = 0; j < nu; ++j) in_u |= ub[j] == b;
            if (!in_u) lane_bits[nl++] = b;
        }
        for (int b = 0; b < n && w < nu + 5; ++b) {
            int uj = -1, lt = -1;
            for (int j = 0; j < nu; ++j)
                if (ub[j] == b) uj = j;
            for (int t2 = 0; t2 < 5; ++t2)
                if (lane_bits[t2] == b) lt = t2;
            if (uj < 0 && lt < 0) continue;
            a.wg[w] = 1u << b;
            a.ws[w] = uj >= 0 ? (1u << (nu - 1 - uj)) * 33u : (1u << lt);
            ++w;
        }
        if (w != nu + 5 || a.wg[0] != 1u || a.wg[4] != 16u) return set_error(QGB_EINVAL, "staged trajectory geometry");
    }
    a.p_dep = k > 0 ? p_dep : 0.0;
    a.seed0 = uint32_t(seed);
    a.seed1 = uint32_t(seed >> 32);
    a.event = event;
    a.nblk = qgb_traj_blocks(n);
    a.log_paulis = pauli_log != nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = dtype == QGB_C64 ? dispatch_gate<float>(sv, gate, kraus, partials, pauli_log, a, st)
                              : dispatch_gate<double>(sv, gate, kraus, partials, pauli_log, a, st);
    if (rc || k == 0) return rc;
    TrajDecideArgs d{};
    d.ntraj = ntraj;
    d.ku = nu;
    d.nblk = a.nblk;
    d.kg = k;
    d.gpos[0] = a.gpos[0];
    d.gpos[1] = k > 1 ? a.gpos[1] : 0;
    d.gamma = gamma;
    d.seed0 = a.seed0;
    d.seed1 = a.seed1;
    d.event = event;
    const unsigned blocks = unsigned((ntraj + 127) / 128);
    if (dtype == QGB_C64)
        traj_decide_kernel<float><<<blocks, 128, 0, st>>>(partials, (float2*)kraus, jump_log, d);
    else
        traj_decide_kernel<double><<<blocks, 128, 0, st>>>(partials, (double2*)kraus, jump_log, d);
    return check_launch("trajectory decide kernel");
}

extern "C" void qgb_philox_uniform(uint32_t event, uint32_t traj, uint32_t stream, uint64_t seed, double* out) {
    *out = qgb::Philox::uniform(event, traj, stream, uint32_t(seed), uint32_t(seed >> 32));
}
