// Dense k-qubit gate application on the 5th-generation tensor cores
// (tcgen05, sm_103a), complex64, k = 4, 5, 6: one read and one write of the
// state per fused block, like dense_reg_kernel, but with the arithmetic moved
// off the FP32 pipes so that 6-qubit blocks (half the HBM passes of 4-qubit
// blocks) still run at memory speed.
//
// Replaces the reference's per-gate `op_action` (tensorQ/statevector_sim.py:124-140)
// for fused blocks of up to six qubits.
//
// Formulation. A group is the 2^k amplitudes that differ only in the target
// bits. For 128 groups at a time the kernel forms the real product
//     Y[128 x 2D] = X[128 x 2D] * W[2D x 2D],     D = 2^k,
// where row g of X holds group g's amplitudes as (re, im) pairs in memory
// order of the target bits, and W is the real form [[Mr, Mi], [-Mi, Mr]] of the
// (row/column permuted) gate matrix. That is 8 * D real flops per amplitude,
// the same count as the complex product.
//
// Precision. kind::f16 multiplies fp16 operands (11 significant bits, the
// tf32 precision at twice its rate and half its tensor-memory footprint), so
// every operand is scaled by a power of two and split as x = hi + lo with
// hi = fp16(x) and lo = fp16(x - hi); Y = Xhi*Wlo + Xlo*Whi + Xhi*Whi with fp32
// accumulation (the dropped Xlo*Wlo term is below 2^-21 relative). Each group
// row gets its own scale 2^s with max |x| 2^s in [2^14, 2^15) (the two warps
// that share a row agree on s through a named barrier), the matrix one scale
// for the launch, so no operand overflows fp16 and only components below
// 2^-24 of their row's largest fall into fp16's subnormal range; the
// accumulator is scaled back in the drain. The result agrees with an fp32 dot
// product to its own rounding level (about 1e-7 relative to the group norm).
//
// Data path per CTA (one CTA per SM; 8 data warps + 1 MMA warp):
//   * a tile is 8192 amplitudes (64 KB): the k target bits and the 13 - k
//     lowest other bits (so runs of >= 128 contiguous amplitudes); the data
//     warps copy tiles into two shared-memory buffers with cp.async in memory
//     order (coalesced whatever the targets), two tiles ahead, 16-byte granules
//     XOR-swizzled by the granule row so that row-wise reads spread over banks;
//   * tensor memory (TMEM) holds, per block of 128 groups, two X buffers (hi
//     and lo rows, the A operands: lane = group row, one 32-bit column per
//     fp16 (re, im) pair) and two fp32 accumulators; tiles alternate between
//     buffer pair 0 and 1 (shared memory, X, accumulator);
//   * shared memory also holds Whi, Wlo as the B operand, K-major, no swizzle:
//     8-row x 16-byte core matrices, K-adjacent cores 128 B apart (leading
//     byte offset) and N-adjacent cores 256 B apart (stride byte offset);
//   * warps w and w+4 share TMEM lane quarter w (groups 32w..32w+31 of each
//     block); warp w+4h reads, scales, splits and stages components
//     [h*D/2, (h+1)*D/2) of its groups, and later drains the same half of the
//     result rows straight to HBM;
//   * unitary ops (UNIT): each group row is rescaled to its input norm after the
//     product, in two phases around the pipeline's CTA-wide barriers;
//   * the MMA warp waits on an mbarrier that the 8 data warps arrive at once a
//     tile's X rows are staged, issues the 3 * (2D/16) MMAs per block
//     (M = 128, N = 2D, K = 16) and commits them to a second mbarrier, which the
//     data warps wait on before draining. So the MMAs of tile i run while the
//     data warps drain tile i - 1 and stage tile i + 1.
// Every wait on the mbarrier is bounded (about 2 s of %globaltimer); a wait
// that runs out sets a device status word read by qgb_check_status, and the
// CTA frees its tensor memory and returns.
#include <cuda_fp16.h>

#include <cstdio>
#include <cstdlib>

#include "tc_common.cuh"

namespace qgb {

__device__ int g_tc_status = 0;




// MODE 0: any op. MODE 1 (unitary op): each group's norm is restored after the
// product. MODE 2 (unitary op, one state): a norm chain across consecutive
// passes, in epochs of kChainEpoch passes -- the pass that starts a chain records
// its input's squared norm as the chain's reference; the last pass of an epoch
// records its output's squared norm; the first pass of the next epoch scales its
// matrix by sqrt(reference / that output), undoing the norm drift of the epoch
// (the tensor cores' round-toward-zero accumulation, ~1e-7 per pass). The passes
// in between run as MODE 0. The norm stays within about one epoch's drift of the
// reference, without the row-wise exchange of MODE 1.
template <int K, int MODE>
__global__ void __launch_bounds__(kTcThreads, 1) dense_tc_kernel(float2* __restrict__ sv, const float2* __restrict__ op,
                                                                 const __grid_constant__ TcArgs a) {
    constexpr bool UNIT = MODE == 1;
    using G = TcGeom<K>;
    constexpr int D = G::D, H = G::H, R = G::R, NB = G::NB, BC = G::BCOLS;
    extern __shared__ unsigned char tc_smem_raw[];
    unsigned char* sb = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 127) & ~uintptr_t(127));
    unsigned char* Bhi = sb;
    unsigned char* Blo = sb + G::B_BYTES;
    unsigned char* tiles_smem = sb + 2 * G::B_BYTES;  // two staged tiles of TILE_BYTES
    unsigned char* stage_smem = tiles_smem + 2 * G::TILE_BYTES;  // output staging, 2 KB per data warp
    __shared__ __align__(8) uint64_t x_full[2];    // data warps -> MMA warp: X of pair p staged (8 arrivals)
    __shared__ __align__(8) uint64_t mma_done[2];  // MMA warp -> data warps: accumulator of pair p complete
    __shared__ uint32_t tmem_slot;
    __shared__ uint32_t wmax_bits;
    __shared__ int row_exp[NB][2][128];    // per block, thread half and row: that half's scale exponent
    __shared__ float row_in[NB][2][128];   // ... that half's squared input norm (unitary ops)
    __shared__ float row_out[2][NB][2][128];  // per buffer pair: that half's squared output norm (unitary ops)
    __shared__ double chain_red[8][2];        // per data warp: squared norms of its inputs and outputs (MODE 2)
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q = warp & 3, h = (warp >> 2) & 1;
    // MODE 2, the pass that opens an epoch: it starts the chain (measures its input)
    // unless the previous epoch left a reference and an output norm; its matrix is
    // scaled by 1 + gcorr = sqrt(ref / out_prev)
    bool chain_start = false;
    float gcorr = 0.f;
    if constexpr (MODE == 0) {
        // a factor f ~ 1 (the trace chain of density matrices): folded into W as w + w (f - 1)
        if (a.scale) gcorr = float(*a.scale - 1.0);
        // the norm chain's later epochs open with this mode (no per-tile work): scale by
        // sqrt(ref / out_prev) and carry the reference on; an epoch that has an output norm
        // but no reference (the buffer was cleared mid-chain) restarts the chain from that norm
        if (a.chain && a.c_head) {
            double chain_ref = 0.0;
            if (a.c_prev >= 0) {
                const double ref = a.chain[2 * a.c_prev], out = a.chain[2 * a.c_prev + 1];
                if (ref > 0.0 && out > 0.0) {
                    chain_ref = ref;
                    gcorr = float(sqrt(ref / out) - 1.0);
                } else if (out > 0.0) {
                    chain_ref = out;
                }
            }
            if (blockIdx.x == 0 && tid == 0) {
                a.chain[2 * a.c_next] = 0.0;
                a.chain[2 * a.c_next + 1] = 0.0;
                a.chain[2 * a.c_cur] = chain_ref;
            }
        }
    }
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
    double acc_in = 0.0, acc_out = 0.0;  // float sums of up to 16 tiles folded into these
    float f_in = 0.f, f_out = 0.f;
    int n_in = 0, n_out = 0;

    // B operand: W = [[Mr, Mi], [-Mi, Mr]] in (output, input) memory order, scaled by 2^sw, split hi/lo;
    // a chain's correction 1 + g (|g| ~ 1e-7) goes into W (w + w g in one rounding), which the split
    // then carries like any other matrix value
    if (tid == 0) wmax_bits = 0;
    __syncthreads();
    const int sw = tc_build_w<K, kTcThreads>(Bhi, Blo, op, a.perm_out, a.perm_in, MODE != 1 ? gcorr : 0.f,
                                             &wmax_bits, tid);
    const float wunscale = exp2i(-sw);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
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
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint64_t step = gridDim.x;
    const uint64_t t0 = blockIdx.x;  // the grid never exceeds the tile count
    const uint64_t ntiles = (a.tiles - t0 + step - 1) / step;

    if (warp == 8) {
        // ---- MMA warp: one thread issues, in tile order, on alternating buffer pairs.
        if (lane == 0) {
            const uint32_t bhi = tc_smem_u32(Bhi), blo = tc_smem_u32(Blo);
            for (uint64_t k = 0; k < ntiles; ++k) {
                const int pb = int(k & 1);
                if (!tc_wait_bounded(tc_smem_u32(&x_full[pb]), uint32_t((k >> 1) & 1))) {
                    atomicExch(&g_tc_status, 1);
                    break;
                }
                tc_fence_after();
#pragma unroll 1
                for (int bk = 0; bk < NB; ++bk) {
                    const uint32_t d = tmem + uint32_t(bk * BC + 2 * R + pb * R);
                    const uint32_t xh = tmem + uint32_t(bk * BC + pb * R), xl = xh + R / 2;
#pragma unroll 1
                    for (int s = 0; s < R / 16; ++s)
                        tc_mma(d, xh + uint32_t(8 * s), b_desc(blo + uint32_t(s * R * 32)), G::IDESC, s > 0);
#pragma unroll 1
                    for (int s = 0; s < R / 16; ++s)
                        tc_mma(d, xl + uint32_t(8 * s), b_desc(bhi + uint32_t(s * R * 32)), G::IDESC, 1);
#pragma unroll 1
                    for (int s = 0; s < R / 16; ++s)
                        tc_mma(d, xh + uint32_t(8 * s), b_desc(bhi + uint32_t(s * R * 32)), G::IDESC, 1);
                }
                tc_commit(tc_smem_u32(&mma_done[pb]));
            }
        }
        __syncwarp();
    } else {
        // ---- data warps
        const uint32_t row = tmem + (uint32_t(32 * q) << 16);  // this warp's lane quarter
        const uint32_t runmask = (1u << a.L) - 1u;
        // Tile-index and global offsets of this thread's rows (the same in every tile).
        uint32_t sug[NB];  // swizzled tile index of this thread's rows (and half)
        uint64_t gg[NB];   // their global offsets
#pragma unroll
        for (int bk = 0; bk < NB; ++bk) {
            const uint32_t r = uint32_t(bk * 128 + 32 * q + lane);
            uint32_t u = 0;
#pragma unroll
            for (int i = 0; i < 13 - K; ++i) u |= ((r >> i) & 1u) << a.pos_g[i];
            sug[bk] = tile_swz(u | (h ? a.ut_h : 0u));
            gg[bk] = uint64_t(u & runmask) + a.hoff[u >> a.L] + (h ? a.hstride : 0);
        }
        // cp.async granule m of this thread: tile index 2 tid + 512 m
        const uint32_t ctid = 2u * uint32_t(tid);
        const uint32_t sctid = tile_swz(ctid);
        const uint64_t gctid = uint64_t(ctid & runmask) + a.hoff[ctid >> a.L];
        auto tile_base = [&](uint64_t t) -> float2* {
            const uint64_t b = t / a.tiles_per_state, tt = t - b * a.tiles_per_state;
            return sv + int64_t(b) * a.sv_stride + insert_zeros(tt, a.tile_bits, 13);
        };
        auto issue_load = [&](uint64_t t, int pb) {
            const float2* base = tile_base(t) + gctid;
            const uint32_t dst0 = tc_smem_u32(tiles_smem + pb * G::TILE_BYTES);
#pragma unroll
            for (int m = 0; m < 4096 / kTcDataThreads; ++m)
                cp_async16(dst0 + 8u * (sctid ^ tile_swz(512u * uint32_t(m))), base + a.g512[m]);
        };
        using Scl = float[NB];
        // Reads this thread's half rows of the tile staged in buffer pb, scales,
        // splits and stages them into X of pair pb; records 2^-s per block and,
        // for a unitary op, the row's squared norm.
        auto store_x = [&](int pb, Scl& unscale, Scl& nin) {
            const float2* T = reinterpret_cast<const float2*>(tiles_smem + pb * G::TILE_BYTES);
            float2 v[NB][H];
#pragma unroll
            for (int bk = 0; bk < NB; ++bk) {
                if (a.vec2) {
#pragma unroll
                    for (int m = 0; m < H / 2; ++m) {
                        const float4 x = *reinterpret_cast<const float4*>(T + (sug[bk] ^ a.uts[2 * m]));
                        v[bk][2 * m] = make_float2(x.x, x.y);
                        v[bk][2 * m + 1] = make_float2(x.z, x.w);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < H; ++j) v[bk][j] = T[sug[bk] ^ a.uts[j]];
                }
                float m = 0.f;
#pragma unroll
                for (int j = 0; j < H; ++j) m = fmaxf(m, fmaxf(fabsf(v[bk][j].x), fabsf(v[bk][j].y)));
                row_exp[bk][h][32 * q + lane] = scale_exp(m);
                if constexpr (UNIT) row_in[bk][h][32 * q + lane] = sumsq8<2 * H>(reinterpret_cast<const float*>(v[bk]));
                if constexpr (MODE == 2)
                    if (chain_start) f_in += sumsq8<2 * H>(reinterpret_cast<const float*>(v[bk]));
            }
            asm volatile("bar.sync %0, 64;" ::"r"(1 + q) : "memory");  // warps q and q + 4 share these rows
#pragma unroll
            for (int bk = 0; bk < NB; ++bk) {
                if constexpr (UNIT) nin[bk] = row_in[bk][0][32 * q + lane] + row_in[bk][1][32 * q + lane];
                const int e0 = row_exp[bk][0][32 * q + lane], e1 = row_exp[bk][1][32 * q + lane];
                const int se = e0 < e1 ? e0 : e1;
                const float f = exp2i(se);
                const unsigned long long f2 = f2pack(f, f);
                unscale[bk] = exp2i(-se);
#pragma unroll
                for (int c0 = 0; c0 < H; c0 += 8) {
                    uint32_t hi[8], lo[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        float xs, ys;
                        f2unpack(f2mul(f2pack(v[bk][c0 + e].x, v[bk][c0 + e].y), f2), xs, ys);
                        split_f16(xs, ys, hi[e], lo[e]);
                    }
                    const uint32_t col = uint32_t(bk * BC + pb * R + h * H + c0);
                    tmem_st8(row + col, hi);
                    tmem_st8(row + col + R / 2, lo);
                }
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            if constexpr (MODE == 2) {
                if (++n_in == 16) {
                    acc_in += double(f_in);
                    f_in = 0.f;
                    n_in = 0;
                }
            }
        };
        // Stores one 16-column chunk (8 components) of this thread's result row.
        auto put16 = [&](float2* p, int c0, const float* r) {
            if (a.vec4) {
                // Rows are runs of >= 4 contiguous components: pass the 32 rows x 8
                // components through this warp's staging area so that 4 lanes write
                // one row's 64 contiguous bytes (whole sectors) and 8 rows go per store.
                // 16-byte pieces are XOR-swizzled by (row / 2) % 4 against bank conflicts.
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
            } else if (a.vec2) {
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    *reinterpret_cast<float4*>(p + a.off[c0 / 2 + 2 * m]) =
                        make_float4(r[4 * m], r[4 * m + 1], r[4 * m + 2], r[4 * m + 3]);
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) p[a.off[c0 / 2 + e]] = make_float2(r[2 * e], r[2 * e + 1]);
            }
        };
        // Non-unitary ops: the accumulator streams to HBM chunk by chunk.
        auto drain = [&](uint64_t t, int pb, const Scl& unscale) {
            float2* base = tile_base(t);
#pragma unroll
            for (int bk = 0; bk < NB; ++bk) {
                float2* p = base + gg[bk];
                const float u = unscale[bk];
                const uint32_t acc = row + uint32_t(bk * BC + 2 * R + pb * R + h * D);
                // the accumulator is 2^(s + sw) times the result: one multiply by su when that
                // power of two is a normal float, else the two factors in turn
                const float su = u * wunscale;
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
                        for (int e = 0; e < 16; ++e) r[e] = (r[e] * wunscale) * u;
                    }
                    if constexpr (MODE == 2)
                        if (a.c_tail) f_out += sumsq8<16>(r);
                    put16(p, c0, r);
                }
            }
            if constexpr (MODE == 2) {
                if (++n_out == 16) {
                    acc_out += double(f_out);
                    f_out = 0.f;
                    n_out = 0;
                }
            }
        };
        // Unitary ops, in two phases so that the two warps sharing a row meet at a
        // barrier the pipeline has anyway: (A) once the tile's MMAs are complete,
        // publish each half-row's squared norm (accumulator units); (B) after the
        // next CTA-wide barrier, reload the accumulator and store every row rescaled
        // to its input norm -- which removes the tensor cores' round-toward-zero
        // shrinkage. The accumulator stays valid until the MMAs of the tile after
        // next, which wait for phase B.
        auto drain_norms = [&](int pb) {
#pragma unroll
            for (int bk = 0; bk < NB; ++bk) {
                const uint32_t acc = row + uint32_t(bk * BC + 2 * R + pb * R + h * D);
                float y[D];
                tmem_ld_row<D>(acc, y);
                row_out[pb][bk][h][32 * q + lane] = sumsq8<D>(y);
            }
        };
        auto drain_rescaled = [&](uint64_t t, int pb, const Scl& unscale, const Scl& nin) {
            float2* base = tile_base(t);
#pragma unroll
            for (int bk = 0; bk < NB; ++bk) {
                float2* p = base + gg[bk];
                const float u = unscale[bk];
                const uint32_t acc = row + uint32_t(bk * BC + 2 * R + pb * R + h * D);
                const float su = u * wunscale;
                const bool one = su >= 1.17549435e-38f && su <= 1.0e38f;
                const float nraw = row_out[pb][bk][0][32 * q + lane] + row_out[pb][bk][1][32 * q + lane];
                // g = sqrt(nin / nout) - 1 to first order (|g| ~ 1e-7, the next term ~ g^2);
                // y = acc su (1 + g) = fma(acc, su g, acc su): the factor 1 + g itself is
                // within an ulp of 1, where fp32 cannot resolve it
                const float nout = one ? (nraw * su) * su : 0.f;
                const float g = nout > 0.f ? (nin[bk] - nout) / (2.f * nout) : 0.f;
                const unsigned long long cg2 = f2pack(su * g, su * g), su2 = f2pack(su, su);
                float y[D];
                tmem_ld_row<D>(acc, y);
#pragma unroll
                for (int c0 = 0; c0 < D; c0 += 16) {
                    float* r = y + c0;
                    if (one) {
#pragma unroll
                        for (int e = 0; e < 16; e += 2) {
                            const unsigned long long v = f2pack(r[e], r[e + 1]);
                            f2unpack(f2fma(v, cg2, f2mul(v, su2)), r[e], r[e + 1]);
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < 16; ++e) r[e] = (r[e] * wunscale) * u;
                    }
                    put16(p, c0, r);
                }
            }
        };

        // Stage k (tile t0 + k step, pair k % 2): wait for its copy, stage its X
        // rows and signal the MMA warp, refill its shared-memory buffer with
        // tile k + 2, then drain tile k - 1 once its MMAs are complete.
        issue_load(t0, 0);
        cp_async_commit();
        if (ntiles > 1) issue_load(t0 + step, 1);
        cp_async_commit();
        bool fail = false;
        Scl sA, sB, nA, nB;
        auto stage = [&](uint64_t k, Scl& sc, Scl& scp, Scl& nc, Scl& ncp, int pc) -> bool {
            const int pn = pc ^ 1;
            cp_async_wait1();                    // this thread's copies of tile k have landed
            if (data_bar_any(fail)) return false;  // ... and everyone's; a failure seen by any thread stops all
            if constexpr (UNIT) {
                // tile k - 2 (pair pc): its norms were published before this barrier; its
                // accumulator and scales are overwritten only after this point
                if (k >= 2) {
                    tc_fence_after();
                    drain_rescaled(t0 + (k - 2) * step, pc, sc, nc);
                }
            }
            store_x(pc, sc, nc);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tc_smem_u32(&x_full[pc]));
            data_bar();                          // every read of buffer pc is done
            if (k + 2 < ntiles) issue_load(t0 + (k + 2) * step, pc);
            cp_async_commit();
            if (k >= 1) {
                if (!tc_wait_bounded(tc_smem_u32(&mma_done[pn]), uint32_t(((k - 1) >> 1) & 1))) {
                    fail = true;
                    if (tid == 0) atomicExch(&g_tc_status, 2);
                } else {
                    tc_fence_after();
                    if constexpr (UNIT)
                        drain_norms(pn);
                    else
                        drain(t0 + (k - 1) * step, pn, scp);
                }
            }
            return true;
        };
        bool live = true;
        for (uint64_t k = 0; live && k < ntiles; k += 2) {
            live = stage(k, sA, sB, nA, nB, 0);
            if (live && k + 1 < ntiles) live = stage(k + 1, sB, sA, nB, nA, 1);
        }
        if (live) {
            const uint64_t k = ntiles - 1;
            const int pl = int(k & 1);
            if constexpr (UNIT) {
                // tile k - 1's phase B, then tile k's phases A and B
                if (!data_bar_any(fail)) {
                    if (k >= 1) {
                        tc_fence_after();
                        drain_rescaled(t0 + (k - 1) * step, pl ^ 1, pl ? sA : sB, pl ? nA : nB);
                    }
                    if (tc_wait_bounded(tc_smem_u32(&mma_done[pl]), uint32_t((k >> 1) & 1))) {
                        tc_fence_after();
                        drain_norms(pl);
                    } else {
                        fail = true;
                        if (tid == 0) atomicExch(&g_tc_status, 2);
                    }
                    if (!data_bar_any(fail)) {
                        tc_fence_after();
                        drain_rescaled(t0 + k * step, pl, pl ? sB : sA, pl ? nB : nA);
                    }
                }
            } else if (!fail) {
                if (tc_wait_bounded(tc_smem_u32(&mma_done[pl]), uint32_t((k >> 1) & 1))) {
                    tc_fence_after();
                    drain(t0 + k * step, pl, pl ? sB : sA);
                } else if (tid == 0) {
                    atomicExch(&g_tc_status, 2);
                }
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
            for (int w = 0; w < 8; ++w) {
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

int g_dense_impl = -1;  // -1: not read yet; 0: CUDA cores only; 1: tensor cores for k = 5, 6; 2: also k = 4

int dense_impl() {
    if (g_dense_impl < 0) {
        const char* e = getenv("QGB_DENSE_IMPL");
        g_dense_impl = 2;
        if (e && (e[0] == '0' || e[0] == 'c')) g_dense_impl = 0;
        if (e && e[0] == '1') g_dense_impl = 1;
    }
    return g_dense_impl;
}

template <int K, int MODE>
int launch_tc(float2* sv, const float2* op, const TcArgs& a, cudaStream_t st) {
    using G = TcGeom<K>;
    static int per_sm = 0;
    if (per_sm == 0) {
        if (cudaFuncSetAttribute(dense_tc_kernel<K, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(G::SMEM)) != cudaSuccess)
            return qgb_host::check_launch("dense_tc attribute");
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dense_tc_kernel<K, MODE>, kTcThreads, G::SMEM) !=
            cudaSuccess)
            return qgb_host::check_launch("dense_tc occupancy");
        per_sm = occ < 1 ? occ : 1;  // each CTA holds all 512 TMEM columns
        if (per_sm < 1) return qgb_host::set_error(QGB_ECUDA, "dense_tc kernel does not fit on an SM");
    }
    const uint64_t cap = uint64_t(qgb_host::sm_count()) * uint64_t(per_sm);
    const unsigned grid = unsigned(a.tiles < cap ? a.tiles : cap);
    dense_tc_kernel<K, MODE><<<grid, kTcThreads, G::SMEM, st>>>(sv, op, a);
    return qgb_host::check_launch("dense_tc kernel");
}

}  // namespace

namespace qgb_host {

int tc_status_read_clear() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, qgb::g_tc_status, sizeof(int)) != cudaSuccess) return -1;
    if (v != 0) {
        const int z = 0;
        cudaMemcpyToSymbol(qgb::g_tc_status, &z, sizeof(int));
    }
    return v;
}

int set_dense_impl(int mode) {
    if (mode < 0 || mode > 2) return set_error(QGB_EINVAL, "dense implementation %d unknown (0, 1, 2)", mode);
    g_dense_impl = mode;
    return QGB_OK;
}

// The geometry of a tensor-core pass (tile bits, group and component offsets,
// permutations) for a dense op of width k on nbits-bit vectors; `sorted` holds
// the target bits ascending, in_bits / out_bits the matrix-order bits of the
// op's columns and rows. Returns QGB_OK or a QGB error.
int build_tc_args(TcArgs& a, int nbits, const int* sorted, const int* in_bits, const int* out_bits, int k,
                  int64_t batch, int64_t sv_stride) {
    a = TcArgs{};
    a.k = k;
    const int D = 1 << k;
    uint64_t scat[1 << QGB_MAX_K];
    for (int j = 0; j < D; ++j) {
        uint64_t o = 0;
        for (int i = 0; i < k; ++i)
            if ((j >> i) & 1) o |= uint64_t(1) << sorted[i];
        scat[j] = o;
    }
    for (int j = 0; j < D / 2; ++j) a.off[j] = scat[j];
    a.hstride = uint64_t(1) << sorted[k - 1];
    for (int c = 0; c < D; ++c) {
        const uint64_t oi = matrix_offset(c, in_bits, k), oo = matrix_offset(c, out_bits, k);
        for (int j = 0; j < D; ++j) {
            if (scat[j] == oi) a.perm_in[j] = c;
            if (scat[j] == oo) a.perm_out[j] = c;
        }
    }
    a.vec2 = sorted[0] == 0 ? 1 : 0;
    a.vec4 = (k >= 2 && sorted[0] == 0 && sorted[1] == 1) ? 1 : 0;
    // tile bits: the targets and the 13 - k lowest other bits
    {
        int nt = 0, ng = 0, ti = 0;
        for (int b = 0; b < nbits && ti < 13; ++b) {
            bool is_t = false;
            for (int j = 0; j < k; ++j) is_t |= sorted[j] == b;
            if (is_t) {
                a.tile_bits[ti++] = b;
                ++nt;
            } else if (ng < 13 - k) {
                a.pos_g[ng++] = ti;
                a.tile_bits[ti++] = b;
            }
        }
        if (ti != 13 || nt != k || ng != 13 - k) return set_error(QGB_EINVAL, "tensor-core tile geometry");
        a.L = 0;
        while (a.L < 13 && a.tile_bits[a.L] == a.L) ++a.L;
        if (a.L < 7) return set_error(QGB_EINVAL, "tensor-core tile run shorter than 128");
        for (int j = 0; j < (1 << (13 - a.L)); ++j) {
            uint64_t o = 0;
            for (int i = 0; i < 13 - a.L; ++i)
                if ((j >> i) & 1) o |= uint64_t(1) << a.tile_bits[a.L + i];
            a.hoff[j] = o;
        }
        int pos_t[QGB_MAX_K];
        for (int j = 0; j < k; ++j)
            for (int i = 0; i < 13; ++i)
                if (a.tile_bits[i] == sorted[j]) pos_t[j] = i;
        for (int j = 0; j < D / 2; ++j) {
            uint32_t u = 0;
            for (int i = 0; i < k - 1; ++i)
                if ((j >> i) & 1) u |= 1u << pos_t[i];
            a.uts[j] = tile_swz(u);
        }
        a.ut_h = 1u << pos_t[k - 1];
        for (int m = 0; m < 16; ++m) {
            const uint32_t u = 512u * uint32_t(m);
            a.g512[m] = uint64_t(u & ((1u << a.L) - 1u)) + a.hoff[u >> a.L];
        }
    }
    a.tiles_per_state = uint64_t(1) << (nbits - 13);  // 8192 amplitudes per tile
    a.tiles = a.tiles_per_state * uint64_t(batch);
    a.sv_stride = batch > 1 ? sv_stride : 0;
    return QGB_OK;
}

// Tensor-core path for a complex64 dense op; returns QGB_EDECLINE (and touches
// nothing) when the op is not one it takes, so that the caller runs the
// CUDA-core kernel instead.
int try_dense_tc(void* sv, const void* op, int nbits, const int* sorted, const int* in_bits, const int* out_bits,
                 int k, int64_t op_stride, int64_t batch, int64_t sv_stride, int unitary, cudaStream_t st,
                 double* chain, int link, const double* scale) {
    const int mode = dense_impl();
    if (scale && unitary != 0) return QGB_EDECLINE;  // a factor goes with plain (MODE 0) passes only
    if (unitary == 2 && (batch > 1 || !chain)) return QGB_EDECLINE;  // the chain follows one state
    if (mode == 0 || k < 4 || k > 6 || (k == 4 && mode < 2)) return QGB_EDECLINE;
    if (nbits < 13) return QGB_EDECLINE;              // fewer than one 8192-amplitude tile
    if (batch > 1 && op_stride != 0) return QGB_EDECLINE;  // one operator for the whole batch
    TcArgs a{};
    // cp.async copies 16-byte granules: the state (and every state of a batch) must start 16-byte aligned
    if ((reinterpret_cast<uintptr_t>(sv) % 16) || (batch > 1 && (sv_stride % 2))) return QGB_EDECLINE;
    {
        const int rc = build_tc_args(a, nbits, sorted, in_bits, out_bits, k, batch, sv_stride);
        if (rc != QGB_OK) return rc;
    }
    a.scale = scale;
    float2* s = static_cast<float2*>(sv);
    const float2* m = static_cast<const float2*>(op);
    if (unitary == 2) {
        // epochs of kChainEpoch passes: the first corrects (and starts the chain), the
        // last measures its output; the passes between run without norm control
        if (link == 0 && cudaMemsetAsync(chain, 0, 6 * sizeof(double), st) != cudaSuccess)
            return check_launch("norm chain reset");
        const int e = link / kChainEpoch, pos = link % kChainEpoch;
        a.chain = chain;
        a.c_head = pos == 0;
        a.c_tail = pos == kChainEpoch - 1;
        a.c_prev = e > 0 ? (e - 1) % 3 : -1;
        a.c_cur = e % 3;
        a.c_next = (e + 1) % 3;
        // the chain's first pass measures its input and every epoch's last pass its output
        // (MODE 2, sums of squares per tile); the other epochs open in MODE 0, which folds
        // the correction into the matrix only
        if ((a.c_head && e == 0) || a.c_tail) {
            switch (k) {
                case 4: return launch_tc<4, 2>(s, m, a, st);
                case 5: return launch_tc<5, 2>(s, m, a, st);
                default: return launch_tc<6, 2>(s, m, a, st);
            }
        }
        if (!a.c_head) a.chain = nullptr;  // a pass inside an epoch: no chain work at all
        unitary = 0;
    }
    switch (k) {
        case 4: return unitary ? launch_tc<4, 1>(s, m, a, st) : launch_tc<4, 0>(s, m, a, st);
        case 5: return unitary ? launch_tc<5, 1>(s, m, a, st) : launch_tc<5, 0>(s, m, a, st);
        default: return unitary ? launch_tc<6, 1>(s, m, a, st) : launch_tc<6, 0>(s, m, a, st);
    }
}

}  // namespace qgb_host

extern "C" int qgb_set_dense_impl(int mode) { return qgb_host::set_dense_impl(mode); }

extern "C" int qgb_get_dense_impl(void) { return dense_impl(); }
