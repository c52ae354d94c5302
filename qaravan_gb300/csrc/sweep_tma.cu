// TMA-staged, double-buffered sweep kernel.
//
// The state is described to the tensor memory accelerator as a 2-D tensor of
// 128-byte rows (16 eight-byte words per row; one complex64 amplitude is one
// word, one complex128 amplitude two). A tile's contiguous runs of 2^L
// amplitudes are loaded with `cp.async.bulk.tensor.2d` into shared memory
// with the hardware 128-byte swizzle -- the same permutation swz<T> applies,
// because every buffer starts on a 1024-byte boundary -- and stored back the
// same way. Each persistent CTA keeps a ring of two or three tile buffers and
// is warp-specialised: warp 0 only issues copies (one per run, spread over
// its lanes) while the other warps run the sweep's ops, so the loads of the
// next tiles and the store of the previous one overlap the ops on the
// current tile. Per buffer, a `full` mbarrier counts the loaded bytes and a
// `done` mbarrier is released by the compute warps; the producer writes a
// done buffer back (bulk group, waited on read side) before refilling it. The
// compute warps synchronise among themselves on named barrier 1.
//
// Every mbarrier wait is bounded (about 2 s of %globaltimer); a wait that runs
// out sets a device status word (read by qgb_check_status), and the CTA stops
// after waiting for its own outstanding stores.
#include <cudaTypedefs.h>

#include "sweep_common.cuh"

namespace qgb {

__device__ int g_sweep_status = 0;

struct TmaGeom {
    uint32_t tile_bytes;        // 2^m * amplitude bytes (multiple of 1024)
    uint32_t chunk_bytes;       // 2^L * amplitude bytes (multiple of 128)
    uint32_t box_rows;          // 128-byte rows per copy (<= 256)
    uint32_t copies_per_chunk;  // chunk_bytes / (128 * box_rows)
    int W;                      // 8-byte words per amplitude
    int NB;                     // tile buffers in the ring (2 or 3)
};

constexpr int kMaxBuffers = 3;

constexpr unsigned long long kWaitNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    return mbar_wait_parity_bounded(bar, parity, kWaitNs);
}

constexpr int kTmaMaxThreads = 32 + 512;  // producer warp + up to 16 compute warps

template <typename T, int KMAX>
__global__ void __maxnreg__(120) sweep_tma_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                   const cplx<T>* __restrict__ mats,
                                                                   const __grid_constant__ SweepArgs a,
                                                                   const __grid_constant__ TmaGeom g) {
    using C = cplx<T>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sb = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int NB = g.NB;
    auto buf = [&](int j) { return reinterpret_cast<C*>(sb + size_t(j) * g.tile_bytes); };
    C* msh = reinterpret_cast<C*>(sb + size_t(NB) * g.tile_bytes);
    const int L = a.sw.low_bits, H = a.sw.n_high, m = L + H;
    const uint32_t nh = 1u << H;
    uint32_t* hrow = reinterpret_cast<uint32_t*>(msh + stage_elems<KMAX>());
    // full[j]: tile bytes landed in buffer j; done[j]: compute warps finished buffer j
    uint64_t* bars = reinterpret_cast<uint64_t*>(hrow + ((nh + 1) & ~1u));
    volatile int* fail_flag = reinterpret_cast<volatile int*>(bars + 2 * kMaxBuffers);
    for (uint32_t h = threadIdx.x; h < nh; h += blockDim.x) {
        uint64_t o = 0;
        for (int j = 0; j < H; ++j) o |= uint64_t((h >> j) & 1u) << a.sw.high_bits[j];
        hrow[h] = uint32_t((o * uint64_t(g.W)) >> 4);
    }
    if (threadIdx.x == 0) {
        for (int j = 0; j < 2 * kMaxBuffers; ++j)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[j])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *fail_flag = 0;
    }
    __syncthreads();
    const uint64_t total = uint64_t(a.batch) * a.tiles;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t bytes_per_copy = g.box_rows * 128u;
    uint64_t* full = bars;
    uint64_t* done = bars + kMaxBuffers;

    auto row0_of = [&](uint64_t w) -> uint64_t {
        const uint64_t b = w / a.tiles, o = w - b * a.tiles;
        uint64_t base = 0;
        for (int j = 0; j < a.n_outer; ++j) base |= ((o >> j) & 1ull) << a.outer_bits[j];
        return ((b * uint64_t(a.sv_stride) + base) * uint64_t(g.W)) >> 4;
    };

    if (warp == 0) {
        // ---------------- producer: every TMA load and store of this CTA
        auto issue_load = [&](uint64_t w, int j) {
            const uint64_t r0 = row0_of(w);
            const uint32_t bar = smem_u32(&full[j]);
            if (lane == 0)
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(g.tile_bytes)
                             : "memory");
            __syncwarp();
            const uint32_t dst0 = smem_u32(buf(j));
            for (uint32_t h = lane; h < nh; h += 32)
                for (uint32_t c = 0; c < g.copies_per_chunk; ++c)
                    asm volatile(
                        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                            dst0 + h * g.chunk_bytes + c * bytes_per_copy),
                        "l"(&tmap), "r"(0), "r"(int(r0 + hrow[h] + c * g.box_rows)), "r"(bar)
                        : "memory");
        };
        auto issue_store = [&](uint64_t w, int j) {
            const uint64_t r0 = row0_of(w);
            const uint32_t src0 = smem_u32(buf(j));
            for (uint32_t h = lane; h < nh; h += 32)
                for (uint32_t c = 0; c < g.copies_per_chunk; ++c)
                    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(&tmap),
                                 "r"(0), "r"(int(r0 + hrow[h] + c * g.box_rows)), "r"(src0 + h * g.chunk_bytes + c * bytes_per_copy)
                                 : "memory");
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        };
        uint32_t dphase = 0;
        bool failed = false;
        uint64_t issued = 0;
        int j = 0;
        for (uint64_t w = blockIdx.x; w < total; w += gridDim.x, ++issued, j = (j + 1 == NB) ? 0 : j + 1) {
            if (issued >= uint64_t(NB)) {
                // buffer j still holds tile issued-NB: wait until it is computed, write it back,
                // and let the store finish reading shared memory before refilling the buffer
                const bool ok = mbar_wait_bounded(smem_u32(&done[j]), (dphase >> j) & 1u);
                dphase ^= 1u << j;
                if (!__all_sync(0xffffffffu, ok)) {
                    failed = true;
                    break;
                }
                issue_store(w - uint64_t(NB) * gridDim.x, j);
                asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                __syncwarp();
            }
            issue_load(w, j);
        }
        // write back the last (up to) NB tiles
        for (uint64_t t = issued >= uint64_t(NB) ? issued - NB : 0; !failed && t < issued; ++t) {
            const int j = int(t % uint64_t(NB));
            const bool ok = mbar_wait_bounded(smem_u32(&done[j]), (dphase >> j) & 1u);
            dphase ^= 1u << j;
            if (!__all_sync(0xffffffffu, ok)) {
                failed = true;
                break;
            }
            issue_store(blockIdx.x + t * uint64_t(gridDim.x), j);
        }
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        if (failed && lane == 0) atomicExch(&g_sweep_status, 2);
    } else {
        // ---------------- compute warps
        const int tid = threadIdx.x - 32, nthr = blockDim.x - 32;
        uint32_t fphase = 0;
        int j = 0;
        for (uint64_t w = blockIdx.x; w < total; w += gridDim.x, j = (j + 1 == NB) ? 0 : j + 1) {
            const bool ok = mbar_wait_bounded(smem_u32(&full[j]), (fphase >> j) & 1u);
            fphase ^= 1u << j;
            if (!ok) *fail_flag = 1;
            ComputeSync::sync(nthr);
            if (*fail_flag) {
                if (tid == 0) atomicExch(&g_sweep_status, 3);
                break;
            }
            apply_ops<T, KMAX, ComputeSync>(buf(j), m, a, mats + int64_t(w / a.tiles) * a.mat_stride, msh, tid,
                                            nthr);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            ComputeSync::sync(nthr);
            if (tid == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&done[j])) : "memory");
        }
    }
}

}  // namespace qgb

using namespace qgb;

namespace {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

template <typename T, int KMAX>
int launch_tma(const CUtensorMap& tm, const void* mats, const SweepArgs& a, const TmaGeom& g, size_t smem,
               cudaStream_t st) {
    auto kern = sweep_tma_kernel<T, KMAX>;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
            return qgb_host::check_launch("tma sweep attribute");
        attr = true;
    }
    static size_t cached_smem[2] = {0, 0};
    static int cached_per_sm[2] = {0, 0};
    int threads = 32 + 256, per_sm = 0;
    for (int pass = 0; pass < 2; ++pass) {
        const int th = 32 + (pass ? 512 : 256);
        if (cached_smem[pass] != smem) {
            int v = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, th, smem) != cudaSuccess)
                return qgb_host::check_launch("tma sweep occupancy");
            cached_smem[pass] = smem;
            cached_per_sm[pass] = v;
        }
        if (pass == 0) {
            per_sm = cached_per_sm[0];
            if (per_sm != 1) break;  // several CTAs per SM: 256 threads each
        } else if (cached_per_sm[1] >= 1) {
            threads = 32 + 512;  // a single resident CTA: give it 16 compute warps
            per_sm = cached_per_sm[1];
        }
    }
    if (per_sm < 1) return 1;
    const uint64_t total = uint64_t(a.batch) * a.tiles;
    uint64_t grid = uint64_t(per_sm) * qgb_host::sm_count();
    if (grid > total) grid = total;
    kern<<<unsigned(grid), threads, smem, st>>>(tm, (const cplx<T>*)mats, a, g);
    return qgb_host::check_launch("tma sweep kernel");
}

}  // namespace

namespace qgb_host {

int launch_sweep_tma(int dtype, void* sv, const void* mats, const SweepArgs& a, int kmax, cudaStream_t st) {
    const int W = dtype == QGB_C64 ? 1 : 2;
    const uint32_t amp_bytes = 8u * W;
    const int L = a.sw.low_bits, H = a.sw.n_high, m = L + H;
    const uint64_t chunk_bytes = (uint64_t(1) << L) * amp_bytes;
    const uint64_t tile_bytes = (uint64_t(1) << m) * amp_bytes;
    if (chunk_bytes < 128 || tile_bytes < 1024) return 1;
    if (a.batch > 1 && (uint64_t(a.sv_stride) * W) % 16) return 1;
    if (dtype != QGB_C64 && kmax > 4) return 1;
    const int kinst = kmax < 2 ? 2 : kmax;
    const uint64_t rows_per_chunk = chunk_bytes / 128;
    const uint64_t box_rows = rows_per_chunk < 256 ? rows_per_chunk : 256;
    const uint64_t stage = kinst >= 3 ? (uint64_t(1) << (2 * (kinst < kStageK ? kinst : kStageK))) : 0;
    const uint64_t nh = uint64_t(1) << H;
    const size_t extra = stage * amp_bytes + 4 * ((nh + 1) & ~1ull) + 16 * kMaxBuffers + 16;
    int NB = 3;
    size_t smem = 1024 + NB * tile_bytes + extra;
    if (smem > 227 * 1024) {
        NB = 2;
        smem = 1024 + NB * tile_bytes + extra;
    }
    if (smem > 227 * 1024) return 1;
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return 1;
    const uint64_t total_amps = uint64_t(a.batch - 1) * uint64_t(a.sv_stride) + (uint64_t(1) << a.n);
    const uint64_t total_rows = total_amps * W / 16;
    if (total_rows >= (uint64_t(1) << 31)) return 1;
    CUtensorMap tm;
    const cuuint64_t gdim[2] = {16, total_rows};
    const cuuint64_t gstride[1] = {128};
    const cuuint32_t box[2] = {16, cuuint32_t(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, sv, gdim, gstride, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(QGB_ECUDA, "cuTensorMapEncodeTiled failed (%d)", int(r));
    TmaGeom g;
    g.tile_bytes = uint32_t(tile_bytes);
    g.chunk_bytes = uint32_t(chunk_bytes);
    g.box_rows = uint32_t(box_rows);
    g.copies_per_chunk = uint32_t(rows_per_chunk / box_rows);
    g.W = W;
    g.NB = NB;
    if (dtype == QGB_C64) {
        switch (kinst) {
            case 2: return launch_tma<float, 2>(tm, mats, a, g, smem, st);
            case 3: return launch_tma<float, 3>(tm, mats, a, g, smem, st);
            case 4: return launch_tma<float, 4>(tm, mats, a, g, smem, st);
            case 5: return launch_tma<float, 5>(tm, mats, a, g, smem, st);
        }
    } else {
        switch (kinst) {
            case 2: return launch_tma<double, 2>(tm, mats, a, g, smem, st);
            case 3: return launch_tma<double, 3>(tm, mats, a, g, smem, st);
            case 4: return launch_tma<double, 4>(tm, mats, a, g, smem, st);
        }
    }
    return 1;
}

int sweep_status_read_clear() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, qgb::g_sweep_status, sizeof(int)) != cudaSuccess) return -1;
    if (v) {
        const int z = 0;
        cudaMemcpyToSymbol(qgb::g_sweep_status, &z, sizeof(int));
    }
    return v;
}

}  // namespace qgb_host
