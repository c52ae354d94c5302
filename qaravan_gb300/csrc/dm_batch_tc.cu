// An uneven batch of noisy density-matrix circuits in one persistent launch
// on the tensor cores.
//
// The reference runs one DensityMatrixSim at a time, every op a contraction
// over the rank-2n tensor of rho (tensorQ/density_matrix_sim.py:38-42, in
// BaseSim.run's loop, core/base_sim.py:30-53). Here every circuit of the batch
// (8..14 qubits: vec(rho) of 16..28 bits, complex64) is compiled on the host
// into fused 6-bit passes (unitary halves and channel superoperators, as the
// single-circuit path), and ONE kernel runs all passes of all circuits:
//
//  * work items are (pass, set of 8192-entry tiles); a CTA takes the next
//    item from an atomic ticket and runs it with dense_tc.cu's pipeline (tiles
//    copied with cp.async two ahead, split-fp16 operands staged into tensor
//    memory, one MMA warp, the drain straight to HBM);
//  * items are ordered pass by pass across circuits (round r holds the r-th
//    pass of every circuit that has one), and an item waits until every item
//    of its circuit's previous pass is done (a per-circuit counter, read with
//    a bounded spin). Every item's dependencies have smaller tickets and were
//    taken by running CTAs, so the smallest unfinished ticket can always
//    proceed: no deadlock, whatever the grid;
//  * the first pass of a circuit reads |0...0><0...0| without touching HBM;
//  * trace chain (CPTP maps keep Tr rho; the tensor cores' round-toward-zero
//    accumulation shrinks it by ~1e-7 per pass): every item of a tail pass
//    stores the diagonal sum of its output tiles in its own slot, the next
//    (head) pass sums its circuit's tail slots in item order and multiplies
//    its matrix by 1 / that trace, as the single-circuit executor does;
//  * the items of a circuit's last pass store their sums of |rho_ij|^2, and a
//    finishing item per circuit (after all passes) writes the circuit's
//    results: trace and Re Tr(rho Z_q) from the diagonal of vec(rho), purity
//    Tr(rho^2) from the slots. Every sum runs in a fixed order (per thread,
//    then a fixed shuffle tree, then warp by warp), so results are bitwise
//    reproducible whichever CTA takes which item.
// Every wait is bounded (about 2 s); a wait that runs out sets a status word
// (qgb_check_status -> QGB_ETIMEOUT) and the CTA stops taking work.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "tc_common.cuh"

namespace qgb {

__device__ int g_dmb_status = 0;

constexpr int kDmbHead = 1, kDmbTail = 2, kDmbLast = 4, kDmbFirst = 8;
constexpr int kDmbMaxQ = 14;  // qubits of a circuit (vec(rho) of 28 bits)

struct DmbPassDev {
    TcArgs a;           // geometry of the pass (k = 6)
    const float2* mat;  // its 64 x 64 complex64 matrix
    int circ;
    int flags;          // kDmb*
    int64_t tail_item0; // head pass: the first item of the circuit's tail pass (its slots)
    int tail_items;     // ... and their count
    int pad;
};

struct DmbCircDev {
    float2* state;  // vec(rho), 4^n complex64
    int n;
    int out_row;
};

struct DmbItemDev {
    int pass;           // a pass item: its pass; a finishing item: the circuit's last pass
    uint32_t need;      // items of the circuit done before this one may start
    uint32_t t0;        // first tile; the item's tiles are t0, t0 + tstride, ... (ntiles of them)
    uint32_t ntiles;    // 0: the circuit's finishing item
    uint32_t tstride;   // the pass's item count: concurrent items of a pass run adjacent tiles,
                        // so the CTAs stream neighbouring memory together (as one grid-strided launch)
    int last_items;     // finishing item: the last pass's items (their purity slots) ...
    int64_t last0;      // ... starting here
};

struct DmbArgs {
    const DmbPassDev* passes;
    const DmbCircDev* circs;
    const DmbItemDev* items;
    int64_t nitems;
    unsigned int* ticket;
    unsigned int* done;  // per circuit
    double* islots;      // per item: its trace (tail pass) or sum of |rho_ij|^2 (last pass)
    double* out;         // per circuit row: trace, purity, Re Tr(rho Z_q)
    int out_cols;
};

__global__ void __launch_bounds__(kTcThreads, 1) dm_batch_tc_kernel(const __grid_constant__ DmbArgs g) {
    constexpr int K = 6;
    using G = TcGeom<K>;
    constexpr int D = G::D, H = G::H, R = G::R;
    static_assert(G::NB == 1, "one 128-row block per tile");
    extern __shared__ unsigned char dmb_smem_raw[];
    unsigned char* sb =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(dmb_smem_raw) + 127) & ~uintptr_t(127));
    unsigned char* Bhi = sb;
    unsigned char* Blo = sb + G::B_BYTES;
    unsigned char* tiles_smem = sb + 2 * G::B_BYTES;
    unsigned char* stage_smem = tiles_smem + 2 * G::TILE_BYTES;
    __shared__ __align__(8) uint64_t x_full[2];
    __shared__ __align__(8) uint64_t mma_done[2];
    __shared__ uint32_t tmem_slot;
    __shared__ uint32_t wmax_bits;
    __shared__ float wunscale_s;
    __shared__ int row_exp[2][128];
    __shared__ __align__(16) TcArgs sA;  // the current pass's geometry
    __shared__ int64_t s_ticket;
    __shared__ int s_fail;
    __shared__ double s_red[8][16];  // per data warp: its partial sums
    __shared__ double s_head;        // a head pass's trace
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q = warp & 3, h = (warp >> 2) & 1;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_u32(&tmem_slot)),
                     "r"(G::NCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 32) {
        for (int p = 0; p < 2; ++p) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 8;" ::"r"(tc_smem_u32(&x_full[p])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem_u32(&mma_done[p])) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid == 0) s_fail = 0;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    int cur_pass = -1;
    uint64_t ubase = 0;  // units (tiles) run by this CTA so far: buffer pair and mbarrier phases continue

    for (;;) {
        if (tid == 0) s_ticket = int64_t(atomicAdd(g.ticket, 1u));
        __syncthreads();
        const int64_t ticket = s_ticket;
        if (ticket >= g.nitems || s_fail) break;
        const DmbItemDev it = g.items[ticket];
        const DmbPassDev& P = g.passes[it.pass];
        const int circ = P.circ;
        const DmbCircDev C = g.circs[circ];
        const int flags = P.flags;
        if (tid == 0) {
            // every item of this circuit's previous pass is done (bounded wait)
            const volatile unsigned int* dn = g.done + circ;
            const unsigned long long t0 = global_ns();
            while (*dn < it.need) {
                __nanosleep(200);
                if (global_ns() - t0 > kTcWaitNs) {
                    atomicExch(&g_dmb_status, 3);
                    s_fail = 1;
                    break;
                }
            }
            __threadfence();  // acquire: the previous pass's output is visible before our loads
        }
        __syncthreads();  // the dependency is met (or the wait gave up) for every thread
        if (s_fail) break;
        if ((flags & kDmbHead) && it.ntiles != 0) {
            // the tail pass's item slots: lane l of warp 0 sums items l, l + 32, ... in order,
            // then a fixed shuffle tree
            if (warp == 0) {
                double tr = 0.0;
                for (int j = lane; j < P.tail_items; j += 32) tr += __ldcg(&g.islots[P.tail_item0 + j]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) tr += __shfl_down_sync(0xffffffffu, tr, o);
                if (lane == 0) s_head = tr;
            }
            __syncthreads();
        }
        if (it.ntiles == 0) {
            // ---- finishing item: the circuit's results from the diagonal and the last pass's slots
            const int n = C.n;
            const uint64_t dim = uint64_t(1) << n;
            double acc[1 + kDmbMaxQ];
#pragma unroll
            for (int j = 0; j <= kDmbMaxQ; ++j) acc[j] = 0.0;
            if (warp < 8) {
                for (uint64_t x = uint64_t(tid); x < dim; x += kTcDataThreads) {
                    const double re = double(__ldcg(reinterpret_cast<const float*>(C.state + x * (dim + 1))));
                    acc[0] += re;
#pragma unroll
                    for (int qq = 0; qq < kDmbMaxQ; ++qq)
                        if (qq < n) acc[1 + qq] += ((x >> (n - 1 - qq)) & 1u) ? -re : re;
                }
#pragma unroll
                for (int j = 0; j <= kDmbMaxQ; ++j) {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_down_sync(0xffffffffu, acc[j], o);
                }
                if (lane == 0) {
#pragma unroll
                    for (int j = 0; j <= kDmbMaxQ; ++j) s_red[warp][j] = acc[j];
                }
            }
            __syncthreads();
            if (tid == 0) {
                double* o = g.out + int64_t(C.out_row) * g.out_cols;
                double pur = 0.0;
                for (int j = 0; j < it.last_items; ++j) pur += __ldcg(&g.islots[it.last0 + j]);
                o[1] = pur;
                for (int j = 0; j <= n; ++j) {
                    double v = 0.0;
                    for (int w = 0; w < 8; ++w) v += s_red[w][j];
                    o[j == 0 ? 0 : 1 + j] = v;
                }
            }
            __syncthreads();
            continue;
        }
        if (it.pass != cur_pass) {
            // the pass's geometry into shared memory, its matrix into the B operand
            {
                const uint32_t* src = reinterpret_cast<const uint32_t*>(&P.a);
                uint32_t* dst = reinterpret_cast<uint32_t*>(&sA);
                for (int w = tid; w < int(sizeof(TcArgs) / 4); w += kTcThreads) dst[w] = src[w];
            }
            float gcorr = 0.f;
            if (flags & kDmbHead) {
                const double tr = s_head;
                if (tr > 0.0) gcorr = float(1.0 / tr - 1.0);
            }
            if (tid == 0) wmax_bits = 0;
            __syncthreads();
            const int sw = tc_build_w<K, kTcThreads>(Bhi, Blo, P.mat, sA.perm_out, sA.perm_in, gcorr, &wmax_bits, tid);
            if (tid == 0) wunscale_s = exp2i(-sw);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            cur_pass = it.pass;
            __syncthreads();
        }
        const uint64_t ntiles = it.ntiles;
        const uint64_t tstr = it.tstride;

        if (warp == 8) {
            // ---- MMA warp
            if (lane == 0) {
                const uint32_t bhi = tc_smem_u32(Bhi), blo = tc_smem_u32(Blo);
                for (uint64_t k = 0; k < ntiles; ++k) {
                    const uint64_t u = ubase + k;
                    const int pb = int(u & 1);
                    if (!tc_wait_bounded(tc_smem_u32(&x_full[pb]), uint32_t((u >> 1) & 1))) {
                        atomicExch(&g_dmb_status, 1);
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = tmem + uint32_t(2 * R + pb * R);
                    const uint32_t xh = tmem + uint32_t(pb * R), xl = xh + R / 2;
#pragma unroll 1
                    for (int s = 0; s < R / 16; ++s)
                        tc_mma(d, xh + uint32_t(8 * s), b_desc(blo + uint32_t(s * R * 32)), G::IDESC, s > 0);
#pragma unroll 1
                    for (int s = 0; s < R / 16; ++s)
                        tc_mma(d, xl + uint32_t(8 * s), b_desc(bhi + uint32_t(s * R * 32)), G::IDESC, 1);
#pragma unroll 1
                    for (int s = 0; s < R / 16; ++s)
                        tc_mma(d, xh + uint32_t(8 * s), b_desc(bhi + uint32_t(s * R * 32)), G::IDESC, 1);
                    tc_commit(tc_smem_u32(&mma_done[pb]));
                }
            }
            __syncwarp();
        } else {
            // ---- data warps
            const uint32_t row = tmem + (uint32_t(32 * q) << 16);
            const uint32_t runmask = (1u << sA.L) - 1u;
            const int n = C.n;
            const uint64_t dmask = (uint64_t(1) << n) - 1;
            uint32_t sug;
            uint64_t gg;
            {
                const uint32_t r = uint32_t(32 * q + lane);
                uint32_t u = 0;
#pragma unroll
                for (int i = 0; i < 13 - K; ++i) u |= ((r >> i) & 1u) << sA.pos_g[i];
                sug = tile_swz(u | (h ? sA.ut_h : 0u));
                gg = uint64_t(u & runmask) + sA.hoff[u >> sA.L] + (h ? sA.hstride : 0);
            }
            const uint32_t ctid = 2u * uint32_t(tid);
            const uint32_t sctid = tile_swz(ctid);
            const uint64_t gctid = uint64_t(ctid & runmask) + sA.hoff[ctid >> sA.L];
            const bool first = (flags & kDmbFirst) != 0;
            // component offsets from their single-bit basis, in registers (both maps are
            // linear: swizzled tile offsets over XOR, flat offsets over OR), instead of a
            // shared-memory table read per component
            uint32_t ub[K - 1], ob[K - 1];  // vec(rho) has at most 28 bits: flat offsets fit 32 bits
#pragma unroll
            for (int i = 0; i < K - 1; ++i) {
                ub[i] = sA.uts[1 << i];
                ob[i] = uint32_t(sA.off[1 << i]);
            }
            auto ut_of = [&](int j) -> uint32_t {
                uint32_t u = 0;
#pragma unroll
                for (int i = 0; i < K - 1; ++i)
                    if ((j >> i) & 1) u ^= ub[i];
                return u;
            };
            auto off_of = [&](int j) -> uint32_t {
                uint32_t o = 0;
#pragma unroll
                for (int i = 0; i < K - 1; ++i)
                    if ((j >> i) & 1) o |= ob[i];
                return o;
            };
            auto tile_off = [&](uint64_t t) -> uint64_t { return insert_zeros(t, sA.tile_bits, 13); };
            auto issue_load = [&](uint64_t t, int pb) {
                const uint32_t dst0 = tc_smem_u32(tiles_smem + pb * G::TILE_BYTES);
                if (first) {
                    // |0...0><0...0|: zeros, and 1 at flat index 0 (tile 0, tile index 0)
                    float4* d4 = reinterpret_cast<float4*>(tiles_smem + pb * G::TILE_BYTES);
#pragma unroll
                    for (int m = 0; m < 4096 / kTcDataThreads; ++m)
                        d4[(sctid ^ tile_swz(512u * uint32_t(m))) >> 1] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (t == 0 && tid == 0) d4[0] = make_float4(1.f, 0.f, 0.f, 0.f);
                    return;
                }
                const float2* base = C.state + tile_off(t) + gctid;
#pragma unroll
                for (int m = 0; m < 4096 / kTcDataThreads; ++m)
                    cp_async16(dst0 + 8u * (sctid ^ tile_swz(512u * uint32_t(m))), base + sA.g512[m]);
            };
            // stage this thread's half row of the tile in pair pb; returns 2^-s of the row
            auto store_x = [&](int pb) -> float {
                const float2* T = reinterpret_cast<const float2*>(tiles_smem + pb * G::TILE_BYTES);
                float2 v[H];
                if (sA.vec2) {
#pragma unroll
                    for (int m = 0; m < H / 2; ++m) {
                        const float4 x = *reinterpret_cast<const float4*>(T + (sug ^ ut_of(2 * m)));
                        v[2 * m] = make_float2(x.x, x.y);
                        v[2 * m + 1] = make_float2(x.z, x.w);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < H; ++j) v[j] = T[sug ^ ut_of(j)];
                }
                float mx = 0.f;
#pragma unroll
                for (int j = 0; j < H; ++j) mx = fmaxf(mx, fmaxf(fabsf(v[j].x), fabsf(v[j].y)));
                row_exp[h][32 * q + lane] = scale_exp(mx);
                asm volatile("bar.sync %0, 64;" ::"r"(1 + q) : "memory");  // warps q and q + 4 share these rows
                const int e0 = row_exp[0][32 * q + lane], e1 = row_exp[1][32 * q + lane];
                const int se = e0 < e1 ? e0 : e1;
                const float f = exp2i(se);
                const unsigned long long f2 = f2pack(f, f);
#pragma unroll
                for (int c0 = 0; c0 < H; c0 += 8) {
                    uint32_t hi[8], lo[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        float xs, ys;
                        f2unpack(f2mul(f2pack(v[c0 + e].x, v[c0 + e].y), f2), xs, ys);
                        split_f16(xs, ys, hi[e], lo[e]);
                    }
                    const uint32_t col = uint32_t(pb * R + h * H + c0);
                    tmem_st8(row + col, hi);
                    tmem_st8(row + col + R / 2, lo);
                }
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                return exp2i(-se);
            };
            auto put16 = [&](float2* p, int c0, const float* r) {
                if (sA.vec4) {
                    float4* st4 = reinterpret_cast<float4*>(stage_smem + warp * 2048);
#pragma unroll
                    for (int m = 0; m < 4; ++m)
                        st4[lane * 4 + (m ^ ((lane >> 1) & 3))] =
                            make_float4(r[4 * m], r[4 * m + 1], r[4 * m + 2], r[4 * m + 3]);
                    __syncwarp();
                    const int pc = lane & 3;
                    const uint32_t opc = ((pc & 1) ? ob[1] : 0u) | ((pc & 2) ? ob[2] : 0u);  // off(2 pc)
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int rho = 8 * i + (lane >> 2);
                        const float4 x = st4[rho * 4 + (pc ^ ((rho >> 1) & 3))];
                        float2* pr = reinterpret_cast<float2*>(
                            __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(p), rho));
                        *reinterpret_cast<float4*>(pr + (off_of(c0 / 2) | opc)) = x;
                    }
                    __syncwarp();
                } else if (sA.vec2) {
#pragma unroll
                    for (int m = 0; m < 4; ++m)
                        *reinterpret_cast<float4*>(p + off_of(c0 / 2 + 2 * m)) =
                            make_float4(r[4 * m], r[4 * m + 1], r[4 * m + 2], r[4 * m + 3]);
                } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e) p[off_of(c0 / 2 + e)] = make_float2(r[2 * e], r[2 * e + 1]);
                }
            };
            const bool tail = (flags & kDmbTail) != 0, last = (flags & kDmbLast) != 0;
            // diagonal entries (ket bits == bra bits): a row can hold one only if its fixed
            // (non-target) bits agree on every ket/bra pair that has no target bit
            uint64_t tbits = sA.hstride;
#pragma unroll
            for (int i = 0; i < K - 1; ++i) tbits |= ob[i];
            const uint64_t freepair = dmask & ~((tbits | (tbits >> n)) & dmask);
            float f_pur = 0.f;
            double acc_pur = 0.0, acc_tr = 0.0;  // this thread's sums, in tile order
            // the result of tile t (pair pb) to HBM, with the trace / purity / Z sums this pass needs
            auto drain = [&](uint64_t t, int pb, float us) {
                const uint64_t ridx = tile_off(t) + gg;  // flat index of this thread's row
                float2* p = C.state + ridx;
                const uint32_t acc = row + uint32_t(2 * R + pb * R + h * D);
                const float wun = wunscale_s;
                const float su = us * wun;
                const bool one = su >= 1.17549435e-38f && su <= 1.0e38f;
                float y[D];
                tmem_ld_row<D>(acc, y);
#pragma unroll
                for (int c0 = 0; c0 < D; c0 += 16) {
                    float* r = y + c0;
                    if (one) {
                        const unsigned long long su2 = f2pack(su, su);
#pragma unroll
                        for (int e = 0; e < 16; e += 2) f2unpack(f2mul(f2pack(r[e], r[e + 1]), su2), r[e], r[e + 1]);
                    } else {
#pragma unroll
                        for (int e = 0; e < 16; ++e) r[e] = (r[e] * wun) * us;
                    }
                    if (last) f_pur += sumsq8<16>(r);
                    if (tail && ((((ridx >> n) ^ ridx) & freepair) == 0)) {
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            const uint64_t idx = ridx + off_of(c0 / 2 + e);
                            if ((((idx >> n) ^ idx) & dmask) == 0) acc_tr += double(r[2 * e]);
                        }
                    }
                    put16(p, c0, r);
                }
                if (last) {
                    acc_pur += double(f_pur);
                    f_pur = 0.f;
                }
            };

            // the dense_tc pipeline over this item's tiles (units ubase + k)
            issue_load(it.t0, int(ubase & 1));
            cp_async_commit();
            if (ntiles > 1) issue_load(it.t0 + tstr, int((ubase + 1) & 1));
            cp_async_commit();
            bool fail = false;
            float usA = 1.f, usB = 1.f;
            for (uint64_t k = 0; k < ntiles; ++k) {
                const uint64_t u = ubase + k;
                const int pc = int(u & 1), pn = pc ^ 1;
                cp_async_wait1();
                if (data_bar_any(fail)) {
                    fail = true;
                    break;
                }
                const float us = store_x(pc);
                if (pc) usB = us;
                else usA = us;
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(tc_smem_u32(&x_full[pc]));
                data_bar();  // every read of buffer pc is done
                if (k + 2 < ntiles) issue_load(it.t0 + (k + 2) * tstr, pc);
                cp_async_commit();
                if (k >= 1) {
                    if (!tc_wait_bounded(tc_smem_u32(&mma_done[pn]), uint32_t(((u - 1) >> 1) & 1))) {
                        fail = true;
                        if (tid == 0) atomicExch(&g_dmb_status, 2);
                    } else {
                        tc_fence_after();
                        drain(it.t0 + (k - 1) * tstr, pn, pn ? usB : usA);
                    }
                }
            }
            if (!fail && ntiles >= 1) {
                const uint64_t u = ubase + ntiles - 1;
                const int pl = int(u & 1);
                if (tc_wait_bounded(tc_smem_u32(&mma_done[pl]), uint32_t((u >> 1) & 1))) {
                    tc_fence_after();
                    drain(it.t0 + (ntiles - 1) * tstr, pl, pl ? usB : usA);
                } else {
                    fail = true;
                    if (tid == 0) atomicExch(&g_dmb_status, 2);
                }
            }
            asm volatile("cp.async.wait_all;" ::: "memory");
            if (fail && lane == 0) s_fail = 1;
            double v = last ? acc_pur : acc_tr;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) s_red[warp][0] = v;
        }
        ubase += ntiles;
        tc_fence_before();
        __syncthreads();  // the item's tiles are all in HBM (or the CTA gives up)
        tc_fence_after();
        if (s_fail) break;
        if (tid == 0) {
            if (flags & (kDmbTail | kDmbLast)) {
                double v = 0.0;  // warp by warp
                for (int w = 0; w < 8; ++w) v += s_red[w][0];
                g.islots[ticket] = v;
            }
            __threadfence();  // release: this item's output before the count that announces it
            atomicAdd(g.done + circ, 1u);
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(G::NCOLS) : "memory");
    }
}

}  // namespace qgb

using namespace qgb;

namespace {

constexpr size_t kDmbSmem = 2 * size_t(TcGeom<6>::B_BYTES) + 2 * size_t(TcGeom<6>::TILE_BYTES) +
                            TcGeom<6>::STAGE_BYTES + 128;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct TableLayout {
    size_t passes, circs, items, total;
};

TableLayout table_layout(int ncirc, int npasses, int64_t nitems) {
    TableLayout t{};
    t.passes = 0;
    t.circs = align256(sizeof(DmbPassDev) * size_t(npasses));
    t.items = t.circs + align256(sizeof(DmbCircDev) * size_t(ncirc));
    t.total = t.items + align256(sizeof(DmbItemDev) * size_t(nitems));
    return t;
}

}  // namespace

namespace qgb_host {

int dmb_status_read_clear() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, qgb::g_dmb_status, sizeof(int)) != cudaSuccess) return -1;
    if (v != 0) {
        const int z = 0;
        cudaMemcpyToSymbol(qgb::g_dmb_status, &z, sizeof(int));
    }
    return v;
}

}  // namespace qgb_host

extern "C" size_t qgb_dm_batch_circuit_bytes(void) { return sizeof(qgb_dm_circuit); }
extern "C" size_t qgb_dm_batch_pass_bytes(void) { return sizeof(qgb_dm_pass); }

// Items of a circuit's pass: its tiles of 8192 entries dealt round-robin to
// min(items_per_pass, tiles / 16) items (at least one): a pass of a large
// circuit is one wave of items_per_pass (the SM count) items, and no item has
// fewer than 16 tiles unless the whole pass has.
constexpr int64_t kDmbMinTiles = 16;
static int64_t items_of(int n, int items_per_pass) {
    const int64_t tiles = int64_t(1) << (2 * n - 13);
    const int64_t by_size = tiles / kDmbMinTiles > 0 ? tiles / kDmbMinTiles : 1;
    return by_size < items_per_pass ? by_size : items_per_pass;
}

static int check_tables(const qgb_dm_circuit* circs, int ncirc, const qgb_dm_pass* passes, int npasses,
                        int items_per_pass) {
    using qgb_host::set_error;
    if (!circs || !passes || ncirc < 1 || npasses < 1) return set_error(QGB_EINVAL, "empty or null tables");
    if (items_per_pass < 1) return set_error(QGB_EINVAL, "items_per_pass %d < 1", items_per_pass);
    int next = 0;
    for (int c = 0; c < ncirc; ++c) {
        const qgb_dm_circuit& cc = circs[c];
        if (cc.n < 7 || cc.n > kDmbMaxQ) return set_error(QGB_EINVAL, "circuit %d: %d qubits outside 7..14", c, cc.n);
        if (!cc.state || (cc.state % 16)) return set_error(QGB_EINVAL, "circuit %d: state missing or misaligned", c);
        if (cc.first_pass != next || cc.n_passes < 1) return set_error(QGB_EINVAL, "circuit %d: pass range", c);
        next += cc.n_passes;
        for (int p = cc.first_pass; p < cc.first_pass + cc.n_passes; ++p) {
            const qgb_dm_pass& ps = passes[p];
            if (ps.circ != c) return set_error(QGB_EINVAL, "pass %d belongs to circuit %d, not %d", p, ps.circ, c);
            if (!ps.mat || (ps.mat % 8)) return set_error(QGB_EINVAL, "pass %d: matrix missing or misaligned", p);
            uint32_t seen = 0;
            for (int j = 0; j < 6; ++j) {
                const int b = ps.bits[j];
                if (b < 0 || b >= 2 * cc.n || ((seen >> b) & 1u))
                    return set_error(QGB_EINVAL, "pass %d: bad bit %d", p, b);
                seen |= 1u << b;
            }
            if (ps.flags & ~15) return set_error(QGB_EINVAL, "pass %d: unknown flags %d", p, ps.flags);
            if (((ps.flags & kDmbFirst) != 0) != (p == cc.first_pass))
                return set_error(QGB_EINVAL, "pass %d: the first-pass flag marks a circuit's first pass", p);
            if (((ps.flags & kDmbLast) != 0) != (p == cc.first_pass + cc.n_passes - 1))
                return set_error(QGB_EINVAL, "pass %d: the last-pass flag marks a circuit's last pass", p);
            if (ps.flags & kDmbHead) {
                // the trace comes from an earlier tail pass of the same circuit
                if (ps.tslot < cc.first_pass || ps.tslot >= p || !(passes[ps.tslot].flags & kDmbTail))
                    return set_error(QGB_EINVAL, "pass %d: trace slot %d is not an earlier tail pass", p, ps.tslot);
            }
        }
    }
    if (next != npasses) return set_error(QGB_EINVAL, "circuits cover %d of %d passes", next, npasses);
    return QGB_OK;
}

extern "C" int64_t qgb_dm_batch_items(const qgb_dm_circuit* circs, int ncirc, int items_per_pass) {
    if (!circs || ncirc < 1 || items_per_pass < 1) return -1;
    int64_t total = ncirc;  // a finishing item per circuit
    for (int c = 0; c < ncirc; ++c) {
        if (circs[c].n < 7 || circs[c].n > 14) return -1;
        total += items_of(circs[c].n, items_per_pass) * circs[c].n_passes;
    }
    return total;
}

extern "C" size_t qgb_dm_batch_table_bytes(int ncirc, int npasses, int64_t nitems) {
    if (ncirc < 1 || npasses < 1 || nitems < 1) return 0;
    return table_layout(ncirc, npasses, nitems).total;
}

extern "C" int qgb_dm_batch_build(void* table, size_t table_bytes, const qgb_dm_circuit* circs, int ncirc,
                                  const qgb_dm_pass* passes, int npasses, int items_per_pass) {
    using qgb_host::set_error;
    int rc = check_tables(circs, ncirc, passes, npasses, items_per_pass);
    if (rc) return rc;
    const int64_t nitems = qgb_dm_batch_items(circs, ncirc, items_per_pass);
    const TableLayout L = table_layout(ncirc, npasses, nitems);
    if (!table || table_bytes < L.total) return set_error(QGB_ESCRATCH, "table needs %zu bytes", L.total);
    unsigned char* base = static_cast<unsigned char*>(table);
    memset(base, 0, L.total);
    DmbPassDev* P = reinterpret_cast<DmbPassDev*>(base + L.passes);
    DmbCircDev* Cd = reinterpret_cast<DmbCircDev*>(base + L.circs);
    DmbItemDev* I = reinterpret_cast<DmbItemDev*>(base + L.items);
    for (int c = 0; c < ncirc; ++c) {
        Cd[c].state = reinterpret_cast<float2*>(circs[c].state);
        Cd[c].n = circs[c].n;
        Cd[c].out_row = circs[c].out_row;
    }
    for (int p = 0; p < npasses; ++p) {
        const qgb_dm_pass& ps = passes[p];
        const int nb = 2 * circs[ps.circ].n;
        int sorted[6];
        for (int j = 0; j < 6; ++j) sorted[j] = ps.bits[j];
        for (int i = 1; i < 6; ++i)
            for (int j = i; j > 0 && sorted[j - 1] > sorted[j]; --j) {
                const int t = sorted[j];
                sorted[j] = sorted[j - 1];
                sorted[j - 1] = t;
            }
        rc = qgb_host::build_tc_args(P[p].a, nb, sorted, ps.bits, ps.bits, 6, 1, 0);
        if (rc) return rc;
        P[p].mat = reinterpret_cast<const float2*>(ps.mat);
        P[p].circ = ps.circ;
        P[p].flags = ps.flags;
    }
    // rounds: the r-th pass of every circuit that has one, in circuit order; items of a pass
    // wait for all items of the circuit's previous pass
    int maxp = 0;
    for (int c = 0; c < ncirc; ++c) maxp = circs[c].n_passes > maxp ? circs[c].n_passes : maxp;
    std::vector<int64_t> item0(size_t(npasses), 0);  // first item of each pass
    int64_t w = 0;
    for (int r = 0; r < maxp; ++r)
        for (int c = 0; c < ncirc; ++c) {
            if (r >= circs[c].n_passes) continue;
            const int64_t per = items_of(circs[c].n, items_per_pass);
            const uint64_t tiles = uint64_t(1) << (2 * circs[c].n - 13);
            item0[size_t(circs[c].first_pass + r)] = w;
            for (int64_t j = 0; j < per; ++j) {
                I[w].pass = circs[c].first_pass + r;
                I[w].need = uint32_t(per * r);
                I[w].t0 = uint32_t(j);
                I[w].tstride = uint32_t(per);
                I[w].ntiles = uint32_t((tiles - uint64_t(j) + uint64_t(per) - 1) / uint64_t(per));
                ++w;
            }
        }
    for (int c = 0; c < ncirc; ++c) {  // finishing items, after every pass of the circuit
        const int64_t per = items_of(circs[c].n, items_per_pass);
        const int lastp = circs[c].first_pass + circs[c].n_passes - 1;
        I[w].pass = lastp;
        I[w].need = uint32_t(per * circs[c].n_passes);
        I[w].t0 = I[w].ntiles = 0;
        I[w].tstride = 1;
        I[w].last0 = item0[size_t(lastp)];
        I[w].last_items = int(per);
        ++w;
    }
    for (int p = 0; p < npasses; ++p)
        if (passes[p].flags & kDmbHead) {
            P[p].tail_item0 = item0[size_t(passes[p].tslot)];
            P[p].tail_items = int(items_of(circs[passes[p].circ].n, items_per_pass));
        }
    return w == nitems ? QGB_OK : set_error(QGB_EINVAL, "item count mismatch");
}

extern "C" size_t qgb_dm_batch_work_bytes(int ncirc, int64_t nitems) {
    if (ncirc < 1 || nitems < 1) return 0;
    return align256(sizeof(unsigned int) * (1 + size_t(ncirc))) + sizeof(double) * size_t(nitems);
}

extern "C" int qgb_dm_batch_run(const void* table, size_t table_bytes, int ncirc, int npasses, int64_t nitems,
                                double* out, int out_rows, int out_cols, void* work, size_t work_bytes, void* stream) {
    using qgb_host::set_error;
    if (!table || !out || !work) return set_error(QGB_EINVAL, "null pointer");
    if (ncirc < 1 || npasses < 1 || nitems < 1) return set_error(QGB_EINVAL, "empty batch");
    const TableLayout L = table_layout(ncirc, npasses, nitems);
    if (table_bytes < L.total) return set_error(QGB_EINVAL, "table of %zu bytes, %zu needed", table_bytes, L.total);
    if (out_cols < 2 + 14 || out_rows < 1) return set_error(QGB_EINVAL, "out needs at least 16 columns");
    const size_t wb = qgb_dm_batch_work_bytes(ncirc, nitems);
    if (work_bytes < wb) return set_error(QGB_ESCRATCH, "work buffer of %zu bytes, %zu needed", work_bytes, wb);
    if ((reinterpret_cast<uintptr_t>(work) % 16) || (reinterpret_cast<uintptr_t>(table) % 16) ||
        (reinterpret_cast<uintptr_t>(out) % 8))
        return set_error(QGB_EINVAL, "table, work or out misaligned");
    cudaStream_t st = (cudaStream_t)stream;
    // counters, trace slots and result rows start at zero (the caller's memory, cleared here)
    if (cudaMemsetAsync(work, 0, wb, st) != cudaSuccess ||
        cudaMemsetAsync(out, 0, sizeof(double) * size_t(out_rows) * size_t(out_cols), st) != cudaSuccess)
        return qgb_host::check_launch("batch counters reset");
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(dm_batch_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDmbSmem)) !=
            cudaSuccess)
            return qgb_host::check_launch("dm batch attribute");
        attr = true;
    }
    const unsigned char* base = static_cast<const unsigned char*>(table);
    DmbArgs a{};
    a.passes = reinterpret_cast<const DmbPassDev*>(base + L.passes);
    a.circs = reinterpret_cast<const DmbCircDev*>(base + L.circs);
    a.items = reinterpret_cast<const DmbItemDev*>(base + L.items);
    a.nitems = nitems;
    unsigned char* wk = static_cast<unsigned char*>(work);
    a.ticket = reinterpret_cast<unsigned int*>(wk);
    a.done = a.ticket + 1;
    a.islots = reinterpret_cast<double*>(wk + align256(sizeof(unsigned int) * (1 + size_t(ncirc))));
    a.out = out;
    a.out_cols = out_cols;
    const int64_t sms = qgb_host::sm_count();
    const unsigned grid = unsigned(nitems < sms ? nitems : sms);  // one CTA per SM: each holds all TMEM columns
    dm_batch_tc_kernel<<<grid, kTcThreads, kDmbSmem, st>>>(a);
    return qgb_host::check_launch("dm batch kernel");
}
