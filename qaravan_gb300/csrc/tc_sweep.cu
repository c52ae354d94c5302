// Several fused blocks per HBM pass on the tensor cores (complex64, 5-qubit
// blocks): the multi-block counterpart of dense_tc.cu.
//
// The reference applies every gate as its own contraction over the state
// (tensorQ/statevector_sim.py:124-140, called gate by gate from
// core/base_sim.py:30-53). dense_tc.cu already fuses gates into 6-qubit
// blocks, one block per read and write of the state; at 0.9 of the copy
// bandwidth per pass, the pass count is what is left. Here a pass takes a tile
// of 8192 amplitudes -- the low L flat bits (L >= 4) times 13 - L chosen high
// bits -- and applies up to four 5-qubit blocks to it in turn, each on five of
// the tile's bits, before the tile goes back to HBM.
//
// Per block the product is the one of dense_tc.cu: for the 256 groups of the
// tile (2^(13-5); a group is the 32 amplitudes that differ in the block's five
// bits), Y[256 x 64] = X[256 x 64] * W[64 x 64] in real form, split-fp16
// operands (x = hi + lo, three kind::f16 MMAs, fp32 accumulation), a
// power-of-two scale per group row and per block matrix.
//
// Data path per CTA (one per SM; 16 data warps + 1 MMA warp -- twice dense_tc.cu's
// data warps, one 128-row block per thread, because the per-block work here is
// latency-bound: stage, MMA and drain of a tile's blocks follow one another):
//   * the CTA takes pairs of tiles (A, B) and interleaves them block by block:
//     units (A, 0), (B, 0), (A, 1), (B, 1), ...; while the MMAs of one unit run,
//     the data warps drain the previous unit and stage the next;
//   * both tiles sit in shared memory (two 64 KB buffers, cp.async in memory
//     order, 16-byte granules swizzled as in dense_tc.cu); a unit reads its
//     group rows from the tile, scales and splits them into tensor memory (the
//     MMA's A operand, buffer pair = the tile's slot), and the drain writes the
//     result rows back into the tile in place (the same positions it read) --
//     except for the tile's last block, whose result goes straight to HBM;
//     once the last block's rows are staged the buffer is free and the copy
//     of the slot's next tile starts, so the load overlaps the last MMAs and
//     drains;
//   * all block matrices of the sweep (W = [[Mr, Mi], [-Mi, Mr]] split hi/lo,
//     16 KB per block) stay in shared memory for the whole launch;
//   * norm chain (MODE 2, unitary sweeps): as dense_tc.cu, per pass -- the
//     first pass of an epoch folds its correction into the first block's
//     matrix, the last pass of an epoch measures its output.
// Every mbarrier wait is bounded (about 2 s); a wait that runs out sets a
// status word (qgb_check_status -> QGB_ETIMEOUT), the data warps agree on the
// failure at their next barrier, and the CTA frees its tensor memory and
// returns.
#include <cstdio>
#include <cstdlib>

#include "tc_common.cuh"

namespace qgb {

__device__ int g_tcs_status = 0;

constexpr int kTcsK = 5;
constexpr int kTcsMaxBlocks = QGB_TCS_MAX_BLOCKS;
constexpr int kTcsDataWarps = 16;
constexpr int kTcsDataThreads = 32 * kTcsDataWarps;
constexpr int kTcsThreads = kTcsDataThreads + 32;  // + the MMA warp
constexpr uint32_t kTcsStageBytes = kTcsDataWarps * 2048;

// Named barriers: 0 the CTA, 1..8 the two warps sharing a (lane quarter, row
// block), 9 the data warps.
__device__ __forceinline__ void tcs_data_bar() { asm volatile("bar.sync 9, 512;" ::: "memory"); }
__device__ __forceinline__ bool tcs_data_bar_any(bool v) {
    uint32_t r;
    asm volatile("{ .reg .pred p, q; setp.ne.u32 p, %1, 0; bar.red.or.pred q, 9, 512, p; selp.u32 %0, 1, 0, q; }"
                 : "=r"(r)
                 : "r"(uint32_t(v))
                 : "memory");
    return r != 0;
}

struct TcsBlock {
    int pos_g[13 - kTcsK];          // tile positions of the group bits, ascending
    int perm_in[1 << kTcsK];        // memory-order input component j -> matrix column
    int perm_out[1 << kTcsK];       // memory-order output component i -> matrix row
    uint32_t uts[1 << (kTcsK - 1)]; // swizzled tile offsets of the low-half components
    uint32_t ub[kTcsK - 1];         // ... of the single low-half bits: uts[j] = XOR of ub[i] over the bits i of j
    uint32_t ut_h;                  // tile offset of the upper half
    int vec2;                       // tile bit 0 is a target: components (2m, 2m+1) adjacent
    int64_t mat;                    // element offset of the block's matrix
};

struct TcsArgs {
    int L;                          // tile bits 0..L-1 are flat bits 0..L-1
    int tile_bits[13];              // flat bit of each tile bit, ascending
    int nblk;
    TcsBlock blk[kTcsMaxBlocks];
    // the last block's result goes to HBM: its global layout
    uint64_t off[1 << (kTcsK - 1)]; // global offsets of the low-half components
    uint64_t hstride;               // global offset of the upper half
    int vec4;                       // flat bits 0 and 1 are targets of the last block
    uint64_t g1024[8];              // global offset of tile index 1024 m
    uint64_t hoff[512];             // global offset of tile bits L..12, indexed by u >> L
    uint64_t pairs;                 // tile pairs per state (tiles 2P and 2P + 1)
    double* chain;                  // norm chain (3 slots of {reference, output}) or null
    int c_prev, c_cur, c_next, c_head, c_tail;
};

template <int MODE>
__global__ void __launch_bounds__(kTcsThreads, 1) tc_sweep_kernel(float2* __restrict__ sv,
                                                                 const float2* __restrict__ mats,
                                                                 const __grid_constant__ TcsArgs a) {
    constexpr int K = kTcsK;
    using G = TcGeom<K>;
    constexpr int D = G::D, H = G::H, R = G::R, NB = G::NB, BC = G::BCOLS;
    extern __shared__ unsigned char tcs_smem_raw[];
    unsigned char* sb =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tcs_smem_raw) + 127) & ~uintptr_t(127));
    unsigned char* wsm = sb;                                          // per block: Bhi, Blo
    unsigned char* tiles_smem = sb + kTcsMaxBlocks * 2 * G::B_BYTES;  // two tiles of TILE_BYTES
    unsigned char* stage_smem = tiles_smem + 2 * G::TILE_BYTES;       // output staging, 2 KB per data warp
    __shared__ __align__(8) uint64_t x_full[2];
    __shared__ __align__(8) uint64_t mma_done[2];
    __shared__ uint32_t tmem_slot;
    __shared__ uint32_t wmax_bits[kTcsMaxBlocks];
    __shared__ float wunscale_s[kTcsMaxBlocks];
    __shared__ int row_exp[NB][2][128];
    __shared__ double chain_red[kTcsDataWarps][2];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // data warp w: TMEM lane quarter q (groups 32q..32q+31 of row block bk), component half h
    const int q = warp & 3, h = (warp >> 2) & 1, bk = (warp >> 3) & 1;
    static_assert(NB == 2, "one 128-row block per data thread");
    const int nblk = a.nblk;

    bool chain_start = false;
    float gcorr = 0.f;
    if constexpr (MODE == 2) {
        if (a.c_head) {
            double chain_ref = 0.0;
            chain_start = true;
            if (a.c_prev >= 0) {
                const double ref = a.chain[2 * a.c_prev], out = a.chain[2 * a.c_prev + 1];
                if (ref > 0.0 && out > 0.0) {
                    chain_start = false;
                    chain_ref = ref;
                    gcorr = float(sqrt(ref / out) - 1.0);
                }
            }
            if (blockIdx.x == 0 && tid == 0) {
                a.chain[2 * a.c_next] = 0.0;
                a.chain[2 * a.c_next + 1] = 0.0;
                if (!chain_start) a.chain[2 * a.c_cur] = chain_ref;
            }
        }
    }
    double acc_in = 0.0, acc_out = 0.0;
    float f_in = 0.f, f_out = 0.f;
    int n_in = 0, n_out = 0;

    // ---- every block's B operand (W in real form, scaled by 2^sw, split hi/lo)
    if (tid < kTcsMaxBlocks) wmax_bits[tid] = 0;
    __syncthreads();
    for (int b = 0; b < nblk; ++b) {
        const float2* op = mats + a.blk[b].mat;
        float m = 0.f;
        for (int p = tid; p < D * D; p += kTcsThreads) {
            const float2 e = op[p];
            m = fmaxf(m, fmaxf(fabsf(e.x), fabsf(e.y)));
        }
        atomicMax(&wmax_bits[b], __float_as_uint(m));
    }
    __syncthreads();
    for (int b = 0; b < nblk; ++b) {
        const float2* op = mats + a.blk[b].mat;
        const int sw = scale_exp(__uint_as_float(wmax_bits[b]));
        const float wscale = exp2i(sw);
        if (tid == 0) wunscale_s[b] = exp2i(-sw);
        unsigned char* Bhi = wsm + size_t(b) * 2 * G::B_BYTES;
        unsigned char* Blo = Bhi + G::B_BYTES;
        const float g = b == 0 ? gcorr : 0.f;
        for (int p = tid; p < D * D; p += kTcsThreads) {
            const int i = p / D, j = p - (p / D) * D;
            const float2 mv = op[a.blk[b].perm_out[i] * D + a.blk[b].perm_in[j]];
            float w[4] = {mv.x * wscale, -mv.y * wscale, mv.y * wscale, mv.x * wscale};
            if (g != 0.f) {
#pragma unroll
                for (int e = 0; e < 4; ++e) w[e] = fmaf(w[e], g, w[e]);
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const uint32_t o = b_off(2 * i + (e >> 1), 2 * j + (e & 1), R);
                const __half hi = __float2half_rn(w[e]);
                *reinterpret_cast<__half*>(Bhi + o) = hi;
                *reinterpret_cast<__half*>(Blo + o) = __float2half_rn(w[e] - __half2float(hi));
            }
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_u32(&tmem_slot)),
                     "r"(G::NCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 32) {
        for (int p = 0; p < 2; ++p) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 16;" ::"r"(tc_smem_u32(&x_full[p])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem_u32(&mma_done[p])) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint64_t step = gridDim.x;
    const uint64_t p0 = blockIdx.x;  // the grid never exceeds the pair count
    const uint64_t npairs = (a.pairs - p0 + step - 1) / step;

    if (warp == kTcsDataWarps) {
        // ---- MMA warp: units in the data warps' order, slot p on buffer pair p. The MMAs of
        // a unit are fully unrolled from two descriptors (a K step adds 2048 bytes, 128 in the
        // descriptor's address field) and alternate between the two row blocks, so that two
        // independent accumulations keep the tensor pipe busy.
        if (lane == 0) {
            uint32_t ph[2] = {0u, 0u};
            bool ok = true;
            const uint32_t wbase = tc_smem_u32(wsm);
            for (uint64_t k = 0; ok && k < npairs; ++k) {
                for (int b = 0; ok && b < nblk; ++b) {
                    const uint64_t dhi = b_desc(wbase + uint32_t(b) * 2u * G::B_BYTES);
                    const uint64_t dlo = b_desc(wbase + uint32_t(b) * 2u * G::B_BYTES + G::B_BYTES);
                    for (int pb = 0; pb < 2; ++pb) {
                        if (!tc_spin_bounded(tc_smem_u32(&x_full[pb]), ph[pb])) {
                            atomicExch(&g_tcs_status, 1);
                            ok = false;
                            break;
                        }
                        ph[pb] ^= 1u;
                        tc_fence_after();
                        const uint32_t d0 = tmem + uint32_t(2 * R + pb * R), d1 = d0 + uint32_t(BC);
                        const uint32_t x0 = tmem + uint32_t(pb * R), x1 = x0 + uint32_t(BC);
                        constexpr uint64_t kStep = uint64_t(R * 32) >> 4;
#pragma unroll
                        for (int s = 0; s < R / 16; ++s) {
                            tc_mma(d0, x0 + uint32_t(8 * s), dlo + s * kStep, G::IDESC, s > 0);
                            tc_mma(d1, x1 + uint32_t(8 * s), dlo + s * kStep, G::IDESC, s > 0);
                        }
#pragma unroll
                        for (int s = 0; s < R / 16; ++s) {
                            tc_mma(d0, x0 + uint32_t(R / 2 + 8 * s), dhi + s * kStep, G::IDESC, 1);
                            tc_mma(d1, x1 + uint32_t(R / 2 + 8 * s), dhi + s * kStep, G::IDESC, 1);
                        }
#pragma unroll
                        for (int s = 0; s < R / 16; ++s) {
                            tc_mma(d0, x0 + uint32_t(8 * s), dhi + s * kStep, G::IDESC, 1);
                            tc_mma(d1, x1 + uint32_t(8 * s), dhi + s * kStep, G::IDESC, 1);
                        }
                        tc_commit(tc_smem_u32(&mma_done[pb]));
                    }
                }
            }
        }
        __syncwarp();
    } else {
        // ---- data warps
        const uint32_t row = tmem + (uint32_t(32 * q) << 16);  // this warp's lane quarter
        const uint32_t runmask = (1u << a.L) - 1u;
        const uint32_t rr = uint32_t(bk * 128 + 32 * q + lane);  // this thread's group row
        const TcsBlock& lb = a.blk[nblk - 1];
        uint64_t gg;  // global offset of this thread's row of the last block (and its half)
        {
            uint32_t u = 0;
#pragma unroll
            for (int i = 0; i < 13 - K; ++i) u |= ((rr >> i) & 1u) << lb.pos_g[i];
            gg = uint64_t(u & runmask) + a.hoff[u >> a.L] + (h ? a.hstride : 0);
        }
        // Per block (up to four, kept in registers and picked by unrolled selects): the
        // swizzled tile index of this thread's row (and half), the component offsets'
        // basis, and whether components pair up (tile bit 0 a target).
        uint32_t rsw[kTcsMaxBlocks], ubs[kTcsMaxBlocks][K - 1];
        uint32_t vec2m = 0;
#pragma unroll
        for (int b = 0; b < kTcsMaxBlocks; ++b) {
            rsw[b] = 0;
#pragma unroll
            for (int i = 0; i < K - 1; ++i) ubs[b][i] = 0;
            if (b < nblk) {
                const TcsBlock& bl = a.blk[b];
                uint32_t u = 0;
#pragma unroll
                for (int i = 0; i < 13 - K; ++i) u |= ((rr >> i) & 1u) << bl.pos_g[i];
                rsw[b] = tile_swz(u | (h ? bl.ut_h : 0u));
#pragma unroll
                for (int i = 0; i < K - 1; ++i) ubs[b][i] = bl.ub[i];
                vec2m |= uint32_t(bl.vec2 != 0) << b;
            }
        }
        // row index and the H component offsets of block b (offset j = XOR of the basis over j's bits)
        auto block_addr = [&](int b, uint32_t (&ut)[H]) -> uint32_t {
            uint32_t r = rsw[0], ub[K - 1];
#pragma unroll
            for (int i = 0; i < K - 1; ++i) ub[i] = ubs[0][i];
#pragma unroll
            for (int c = 1; c < kTcsMaxBlocks; ++c)
                if (b == c) {
                    r = rsw[c];
#pragma unroll
                    for (int i = 0; i < K - 1; ++i) ub[i] = ubs[c][i];
                }
            ut[0] = 0;
#pragma unroll
            for (int i = 0; i < K - 1; ++i)
#pragma unroll
                for (int j = 1 << i; j < (2 << i); ++j) ut[j] = ut[j - (1 << i)] ^ ub[i];
            return r;
        };
        const uint32_t ctid = 2u * uint32_t(tid);
        const uint32_t sctid = tile_swz(ctid);
        const uint64_t gctid = uint64_t(ctid & runmask) + a.hoff[ctid >> a.L];
        auto tile_base = [&](uint64_t t) -> float2* { return sv + insert_zeros(t, a.tile_bits, 13); };
        auto issue_load = [&](uint64_t t, int pb) {
            const float2* base = tile_base(t) + gctid;
            const uint32_t dst0 = tc_smem_u32(tiles_smem + pb * G::TILE_BYTES);
#pragma unroll
            for (int m = 0; m < 4096 / kTcsDataThreads; ++m)
                cp_async16(dst0 + 8u * (sctid ^ tile_swz(1024u * uint32_t(m))), base + a.g1024[m]);
        };
        // Reads this thread's half row of block b from tile slot pb, scales, splits
        // and stages it into X of buffer pair pb; returns 2^-s of the row.
        auto store_x = [&](int pb, int b) -> float {
            const float2* T = reinterpret_cast<const float2*>(tiles_smem + pb * G::TILE_BYTES);
            uint32_t ut[H];
            const uint32_t sug = block_addr(b, ut);
            float2 v[H];
            if ((vec2m >> b) & 1u) {
#pragma unroll
                for (int m = 0; m < H / 2; ++m) {
                    const float4 x = *reinterpret_cast<const float4*>(T + (sug ^ ut[2 * m]));
                    v[2 * m] = make_float2(x.x, x.y);
                    v[2 * m + 1] = make_float2(x.z, x.w);
                }
            } else {
#pragma unroll
                for (int j = 0; j < H; ++j) v[j] = T[sug ^ ut[j]];
            }
            // largest |component|: a tree of three-input maxima
            float mq[H / 2];
#pragma unroll
            for (int j = 0; j < H / 2; ++j)
                mq[j] = fmaxf(fmaxf(fabsf(v[2 * j].x), fabsf(v[2 * j].y)), fmaxf(fabsf(v[2 * j + 1].x), fabsf(v[2 * j + 1].y)));
#pragma unroll
            for (int w = H / 4; w >= 1; w >>= 1)
#pragma unroll
                for (int j = 0; j < w; ++j) mq[j] = fmaxf(mq[j], mq[j + w]);
            const float mx = mq[0];
            row_exp[bk][h][32 * q + lane] = scale_exp(mx);
            if constexpr (MODE == 2)
                if (chain_start && b == 0) f_in += sumsq8<2 * H>(reinterpret_cast<const float*>(v));
            asm volatile("bar.sync %0, 64;" ::"r"(1 + q + 4 * bk) : "memory");  // warps sharing these rows
            const int e0 = row_exp[bk][0][32 * q + lane], e1 = row_exp[bk][1][32 * q + lane];
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
                const uint32_t col = uint32_t(bk * BC + pb * R + h * H + c0);
                tmem_st8(row + col, hi);
                tmem_st8(row + col + R / 2, lo);
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            if constexpr (MODE == 2) {
                if (b == 0 && ++n_in == 16) {
                    acc_in += double(f_in);
                    f_in = 0.f;
                    n_in = 0;
                }
            }
            return exp2i(-se);
        };
        // This thread's half row of the accumulator of buffer pair pb, unscaled.
        auto load_acc = [&](int pb, float us, float wun, float (&y)[D]) {
            const uint32_t acc = row + uint32_t(bk * BC + 2 * R + pb * R + h * D);
            const float su = us * wun;
            tmem_ld_row<D>(acc, y);
            if (su >= 1.17549435e-38f && su <= 1.0e38f) {
                const unsigned long long su2 = f2pack(su, su);
#pragma unroll
                for (int e = 0; e < D; e += 2) f2unpack(f2mul(f2pack(y[e], y[e + 1]), su2), y[e], y[e + 1]);
            } else {  // the power of two is not a normal float: the two factors in turn
#pragma unroll
                for (int e = 0; e < D; ++e) y[e] = (y[e] * wun) * us;
            }
        };
        // A block's result back into its tile slot, in place (not the last block).
        auto drain_smem = [&](int pb, int b, float us) {
            float2* T = reinterpret_cast<float2*>(tiles_smem + pb * G::TILE_BYTES);
            uint32_t ut[H];
            const uint32_t sug = block_addr(b, ut);
            float y[D];
            load_acc(pb, us, wunscale_s[b], y);
            if ((vec2m >> b) & 1u) {
#pragma unroll
                for (int m = 0; m < H / 2; ++m)
                    *reinterpret_cast<float4*>(T + (sug ^ ut[2 * m])) =
                        make_float4(y[4 * m], y[4 * m + 1], y[4 * m + 2], y[4 * m + 3]);
            } else {
#pragma unroll
                for (int j = 0; j < H; ++j) T[sug ^ ut[j]] = make_float2(y[2 * j], y[2 * j + 1]);
            }
        };
        // Stores one 16-column chunk (8 components) of this thread's result row (the last block).
        auto put16 = [&](float2* p, int c0, const float* r) {
            if (a.vec4) {
                // rows are runs of >= 4 contiguous components: the warp's 32 rows x 8 components
                // pass through its staging area so that 4 lanes write one row's 64 contiguous bytes
                float4* st4 = reinterpret_cast<float4*>(stage_smem + warp * 2048);
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    st4[lane * 4 + (m ^ ((lane >> 1) & 3))] = make_float4(r[4 * m], r[4 * m + 1], r[4 * m + 2], r[4 * m + 3]);
                __syncwarp();
                const int pc = lane & 3;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int rho = 8 * i + (lane >> 2);
                    const float4 x = st4[rho * 4 + (pc ^ ((rho >> 1) & 3))];
                    float2* pr = reinterpret_cast<float2*>(
                        __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(p), rho));
                    *reinterpret_cast<float4*>(pr + a.off[c0 / 2 + 2 * pc]) = x;
                }
                __syncwarp();
            } else if (lb.vec2) {
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    *reinterpret_cast<float4*>(p + a.off[c0 / 2 + 2 * m]) =
                        make_float4(r[4 * m], r[4 * m + 1], r[4 * m + 2], r[4 * m + 3]);
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) p[a.off[c0 / 2 + e]] = make_float2(r[2 * e], r[2 * e + 1]);
            }
        };
        // The last block's result straight to HBM.
        auto drain_global = [&](uint64_t t, int pb, float us) {
            float2* p = tile_base(t) + gg;
            float y[D];
            load_acc(pb, us, wunscale_s[nblk - 1], y);
#pragma unroll
            for (int c0 = 0; c0 < D; c0 += 16) {
                if constexpr (MODE == 2)
                    if (a.c_tail) f_out += sumsq8<16>(y + c0);
                put16(p, c0, y + c0);
            }
            if constexpr (MODE == 2) {
                if (++n_out == 16) {
                    acc_out += double(f_out);
                    f_out = 0.f;
                    n_out = 0;
                }
            }
        };

        // Units in order (pair k, block b, slot pb); unit i stages, then drains unit i - 1
        // (the other slot) once its MMAs are complete. The slot's copy for the next pair
        // starts as soon as its last block is staged.
        issue_load(2 * p0, 0);
        cp_async_commit();
        issue_load(2 * p0 + 1, 1);
        cp_async_commit();
        bool fail = false;
        uint32_t dph[2] = {0u, 0u};  // mma_done phase per slot
        float us0 = 1.f, us1 = 1.f;  // row unscale of the unit in flight per slot
        int prev_pb = -1, prev_b = 0;
        uint64_t prev_t = 0;
        for (uint64_t k = 0; k < npairs && !fail; ++k) {
            const uint64_t pr = p0 + k * step;
            for (int b = 0; b < nblk && !fail; ++b) {
                for (int pb = 0; pb < 2; ++pb) {
                    if (b == 0) {
                        // this slot's tile has landed: slot 0 waits for its group (slot 1's is younger);
                        // slot 1 for its own -- younger still is slot 0's next tile when a sweep has
                        // one block (its copy starts as soon as that block is staged)
                        if (pb == 0 || nblk == 1) cp_async_wait1();
                        else asm volatile("cp.async.wait_group 0;" ::: "memory");
                    }
                    // everyone's copies landed / the previous drain into this slot is complete;
                    // a failure seen by any data thread stops all of them
                    if (tcs_data_bar_any(fail)) {
                        fail = true;
                        break;
                    }
                    const float us = store_x(pb, b);
                    if (pb) us1 = us;
                    else us0 = us;
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(tc_smem_u32(&x_full[pb]));
                    if (b == nblk - 1) {
                        tcs_data_bar();  // every read of this slot's tile is done: copy the slot's next tile
                        if (k + 1 < npairs) issue_load(2 * (pr + step) + pb, pb);
                        cp_async_commit();
                    }
                    if (prev_pb >= 0) {
                        if (!tc_spin_bounded(tc_smem_u32(&mma_done[prev_pb]), dph[prev_pb])) {
                            fail = true;
                            if (tid == 0) atomicExch(&g_tcs_status, 2);
                        } else {
                            dph[prev_pb] ^= 1u;
                            tc_fence_after();
                            const float pus = prev_pb ? us1 : us0;
                            if (prev_b == nblk - 1) drain_global(prev_t, prev_pb, pus);
                            else drain_smem(prev_pb, prev_b, pus);
                        }
                    }
                    prev_pb = pb;
                    prev_b = b;
                    prev_t = 2 * pr + pb;
                }
            }
        }
        if (!fail && prev_pb >= 0) {
            if (tc_spin_bounded(tc_smem_u32(&mma_done[prev_pb]), dph[prev_pb])) {
                tc_fence_after();
                drain_global(prev_t, prev_pb, prev_pb ? us1 : us0);
            } else if (tid == 0) {
                atomicExch(&g_tcs_status, 2);
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        if constexpr (MODE == 2) {
            acc_in += double(f_in);
            acc_out += double(f_out);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                acc_in += __shfl_down_sync(0xffffffffu, acc_in, o);
                acc_out += __shfl_down_sync(0xffffffffu, acc_out, o);
            }
            if (lane == 0) {
                chain_red[warp][0] = acc_in;
                chain_red[warp][1] = acc_out;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if constexpr (MODE == 2) {
        if (tid == 0) {
            double in = 0.0, out = 0.0;
            for (int w = 0; w < kTcsDataWarps; ++w) {
                in += chain_red[w][0];
                out += chain_red[w][1];
            }
            if (chain_start) atomicAdd(&a.chain[2 * a.c_cur], in);
            if (a.c_tail) atomicAdd(&a.chain[2 * a.c_cur + 1], out);
        }
    }
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(G::NCOLS) : "memory");
    }
}

}  // namespace qgb

using namespace qgb;

namespace {

constexpr size_t kTcsSmem = size_t(kTcsMaxBlocks) * 2 * TcGeom<kTcsK>::B_BYTES + 2 * size_t(TcGeom<kTcsK>::TILE_BYTES) +
                            kTcsStageBytes + 128;

template <int MODE>
int launch_tcs(float2* sv, const float2* mats, const TcsArgs& a, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(tc_sweep_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTcsSmem)) !=
            cudaSuccess)
            return qgb_host::check_launch("tc_sweep attribute");
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tc_sweep_kernel<MODE>, kTcsThreads, kTcsSmem) !=
            cudaSuccess)
            return qgb_host::check_launch("tc_sweep occupancy");
        if (occ < 1) return qgb_host::set_error(QGB_ECUDA, "tc_sweep kernel does not fit on an SM");
        attr = true;
    }
    const uint64_t cap = uint64_t(qgb_host::sm_count());  // one CTA per SM: each holds all 512 TMEM columns
    const unsigned grid = unsigned(a.pairs < cap ? a.pairs : cap);
    tc_sweep_kernel<MODE><<<grid, kTcsThreads, kTcsSmem, st>>>(sv, mats, a);
    return qgb_host::check_launch("tc_sweep kernel");
}

}  // namespace

namespace qgb_host {

int tcs_status_read_clear() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, qgb::g_tcs_status, sizeof(int)) != cudaSuccess) return -1;
    if (v != 0) {
        const int z = 0;
        cudaMemcpyToSymbol(qgb::g_tcs_status, &z, sizeof(int));
    }
    return v;
}

}  // namespace qgb_host

extern "C" size_t qgb_tc_sweep_bytes(void) { return sizeof(qgb_tc_sweep); }

extern "C" int qgb_apply_tc_sweep(void* sv, int dtype, int n, const qgb_tc_sweep* sweep, const void* mats,
                                  double* chain, int link, void* stream) {
    using qgb_host::set_error;
    constexpr int K = kTcsK, D = 1 << K;
    if (!sv || !sweep || !mats) return set_error(QGB_EINVAL, "null pointer");
    if (dtype != QGB_C64) return set_error(QGB_EINVAL, "tensor-core sweeps take complex64 states");
    if (n < 14 || n > QGB_MAX_QUBITS) return set_error(QGB_EINVAL, "tensor-core sweeps need 14..%d qubits (n=%d)", QGB_MAX_QUBITS, n);
    if (reinterpret_cast<uintptr_t>(sv) % 16) return set_error(QGB_EINVAL, "state pointer must be 16-byte aligned");
    if (reinterpret_cast<uintptr_t>(mats) % 8) return set_error(QGB_EINVAL, "matrix buffer misaligned");
    if (link < 0) return set_error(QGB_EINVAL, "chain link %d < 0", link);
    const qgb_tc_sweep& sw = *sweep;
    const int L = sw.low_bits, Hn = 13 - L;
    if (L < 4 || L > 13) return set_error(QGB_EINVAL, "low_bits %d outside 4..13", L);
    if (sw.n_blocks < 1 || sw.n_blocks > kTcsMaxBlocks)
        return set_error(QGB_EINVAL, "n_blocks %d outside 1..%d", sw.n_blocks, kTcsMaxBlocks);
    TcsArgs a{};
    a.L = L;
    for (int i = 0; i < L; ++i) a.tile_bits[i] = i;
    int prev = L - 1;
    for (int hh = 0; hh < Hn; ++hh) {
        const int b = sw.high_bits[hh];
        if (b <= prev || b >= n) return set_error(QGB_EINVAL, "high bits must be ascending, >= low_bits and < n");
        a.tile_bits[L + hh] = b;
        prev = b;
    }
    for (int j = 0; j < (1 << Hn); ++j) {
        uint64_t o = 0;
        for (int i = 0; i < Hn; ++i)
            if ((j >> i) & 1) o |= uint64_t(1) << a.tile_bits[L + i];
        a.hoff[j] = o;
    }
    for (int m = 0; m < 8; ++m) {
        const uint32_t u = 1024u * uint32_t(m);
        a.g1024[m] = uint64_t(u & ((1u << L) - 1u)) + a.hoff[u >> L];
    }
    a.nblk = sw.n_blocks;
    for (int b = 0; b < sw.n_blocks; ++b) {
        TcsBlock& bl = a.blk[b];
        const int* pos = sw.block_pos[b];  // tile position of matrix bit K-1-j
        uint32_t seen = 0;
        for (int j = 0; j < K; ++j) {
            if (pos[j] < 0 || pos[j] > 12 || ((seen >> pos[j]) & 1u))
                return set_error(QGB_EINVAL, "block %d has a bad tile bit %d", b, pos[j]);
            seen |= 1u << pos[j];
        }
        if (sw.block_mat[b] < 0) return set_error(QGB_EINVAL, "block %d has a negative matrix offset", b);
        bl.mat = sw.block_mat[b];
        int sorted[K];
        for (int j = 0; j < K; ++j) sorted[j] = pos[j];
        for (int i = 1; i < K; ++i)
            for (int j = i; j > 0 && sorted[j - 1] > sorted[j]; --j) {
                const int t = sorted[j];
                sorted[j] = sorted[j - 1];
                sorted[j - 1] = t;
            }
        int ng = 0;
        for (int p = 0; p < 13; ++p)
            if (!((seen >> p) & 1u)) bl.pos_g[ng++] = p;
        // memory-order component j (bit i of j <-> tile bit sorted[i]) against matrix index c
        // (bit K-1-jj of c <-> tile bit pos[jj])
        uint32_t scat[D];
        for (int j = 0; j < D; ++j) {
            uint32_t o = 0;
            for (int i = 0; i < K; ++i)
                if ((j >> i) & 1) o |= 1u << sorted[i];
            scat[j] = o;
        }
        for (int c = 0; c < D; ++c) {
            uint32_t o = 0;
            for (int jj = 0; jj < K; ++jj)
                if ((c >> (K - 1 - jj)) & 1) o |= 1u << pos[jj];
            for (int j = 0; j < D; ++j)
                if (scat[j] == o) bl.perm_in[j] = bl.perm_out[j] = c;
        }
        for (int j = 0; j < D / 2; ++j) bl.uts[j] = tile_swz(scat[j]);
        for (int i = 0; i < K - 1; ++i) bl.ub[i] = tile_swz(1u << sorted[i]);
        bl.ut_h = 1u << sorted[K - 1];
        bl.vec2 = sorted[0] == 0 ? 1 : 0;
        if (b == sw.n_blocks - 1) {
            // global offsets of the last block's components (tile offset -> flat offset, linear)
            auto flat = [&](uint32_t u) {
                return uint64_t(u & ((1u << L) - 1u)) + a.hoff[u >> L];
            };
            for (int j = 0; j < D / 2; ++j) a.off[j] = flat(scat[j]);
            a.hstride = flat(bl.ut_h);
            a.vec4 = (a.tile_bits[sorted[0]] == 0 && a.tile_bits[sorted[1]] == 1) ? 1 : 0;
        }
    }
    a.pairs = uint64_t(1) << (n - 14);
    cudaStream_t st = (cudaStream_t)stream;
    float2* s = static_cast<float2*>(sv);
    const float2* m = static_cast<const float2*>(mats);
    if (chain) {
        if (link == 0 && cudaMemsetAsync(chain, 0, 6 * sizeof(double), st) != cudaSuccess)
            return qgb_host::check_launch("norm chain reset");
        const int e = link / kChainEpoch, pos = link % kChainEpoch;
        a.chain = chain;
        a.c_head = pos == 0;
        a.c_tail = pos == kChainEpoch - 1;
        a.c_prev = e > 0 ? (e - 1) % 3 : -1;
        a.c_cur = e % 3;
        a.c_next = (e + 1) % 3;
        if (a.c_head || a.c_tail) return launch_tcs<2>(s, m, a, st);
    }
    return launch_tcs<0>(s, m, a, st);
}
