// C ABI plumbing: version, thread-local last error, launch checks, the device
// status word of bounded waits.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "sweep_common.cuh"

namespace qgb {
__device__ int g_status = 0;

// The library's bounded waits, made to run out on purpose: one warp waits on
// a shared-memory mbarrier (mode 0: it expects one arrival that nobody makes;
// mode 2: lane 0 arrives first, so the wait completes) or on a global flag
// that nothing sets (mode 1), with the given limit; a wait that gives up
// records its code in the status word (3: mbarrier, 4: flag) and the kernel
// returns. Nothing else is touched and nothing stays in flight.
__global__ void wait_probe_kernel(int mode, unsigned long long limit_ns, const int* flag) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = uint32_t(__cvta_generic_to_shared(&bar));
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (mode == 1) {
        if (threadIdx.x == 0 && !flag_wait_bounded(flag, 1, limit_ns)) atomicExch(&g_status, 4);
        return;
    }
    if (mode == 2 && threadIdx.x == 0) {
        uint64_t state;
        asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];" : "=l"(state) : "r"(b) : "memory");
        (void)state;
    }
    __syncwarp();
    const bool ok = mbar_wait_parity_bounded(b, 0, limit_ns);
    if (!ok && threadIdx.x == 0) atomicExch(&g_status, 3);
}
}

namespace {
thread_local char g_last_error[512] = "";
}

namespace qgb_host {

int set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

int check_launch(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(QGB_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    return QGB_OK;
}

int sm_count() {
    static int cached = 0;
    if (cached == 0) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            cached = v;
        else
            cached = 148;
    }
    return cached;
}

}  // namespace qgb_host

extern "C" int qgb_abi_version(void) { return QGB_ABI_VERSION; }

extern "C" const char* qgb_last_error(void) { return g_last_error; }

extern "C" int qgb_wait_probe(int mode, unsigned long long limit_ns, const int* flag, void* stream) {
    if (mode < 0 || mode > 2) return qgb_host::set_error(QGB_EINVAL, "wait probe mode %d unknown (0, 1, 2)", mode);
    if (mode == 1 && (!flag || (reinterpret_cast<uintptr_t>(flag) % sizeof(int))))
        return qgb_host::set_error(QGB_EINVAL, "wait probe flag missing or misaligned");
    if (limit_ns > 10000000000ull) return qgb_host::set_error(QGB_EINVAL, "wait probe limit above 10 s");
    qgb::wait_probe_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(mode, limit_ns, flag);
    return qgb_host::check_launch("wait probe");
}

namespace qgb {
// Peak rate of the FMA pipe of one precision: 8 independent chains of fused
// multiply-adds per thread (so the pipe, not the dependency latency, bounds
// it); the sum is stored only under a condition that never holds, which keeps
// the chains alive without memory traffic.
template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T* out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = T(threadIdx.x + j) * T(1e-3);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
    }
    T s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    if (s == T(-1.2345e-7)) out[blockIdx.x] = s;
}

// The same chains as packed pairs (fma.rn.f32x2: one instruction, two float FMAs).
__global__ void __launch_bounds__(256) fma_probe_f32x2_kernel(float* out, int iters, float a, float b) {
    unsigned long long x[8], a2, b2;
    asm("mov.b64 %0, {%1, %1};" : "=l"(a2) : "f"(a));
    asm("mov.b64 %0, {%1, %1};" : "=l"(b2) : "f"(b));
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float v = float(threadIdx.x + j) * 1e-3f;
        asm("mov.b64 %0, {%1, %2};" : "=l"(x[j]) : "f"(v), "f"(v + 1.f));
    }
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[j]) : "l"(a2), "l"(b2));
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        float u, v;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(u), "=f"(v) : "l"(x[j]));
        s += u + v;
    }
    if (s == -1.2345e-7f) out[blockIdx.x] = s;
}
}  // namespace qgb

extern "C" int qgb_fma_probe(int precision, int iters, int blocks_per_sm, void* out, void* stream) {
    if (precision < 0 || precision > 2 || iters < 1 || blocks_per_sm < 1 || blocks_per_sm > 32 || !out)
        return qgb_host::set_error(QGB_EINVAL, "fma probe arguments invalid");
    const unsigned grid = unsigned(qgb_host::sm_count() * blocks_per_sm);
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == 0) qgb::fma_probe_kernel<float><<<grid, 256, 0, st>>>((float*)out, iters, 0.9999999f, 1e-7f);
    else if (precision == 1) qgb::fma_probe_kernel<double><<<grid, 256, 0, st>>>((double*)out, iters, 0.9999999999, 1e-12);
    else qgb::fma_probe_f32x2_kernel<<<grid, 256, 0, st>>>((float*)out, iters, 0.9999999f, 1e-7f);
    return qgb_host::check_launch("fma probe");
}

extern "C" int qgb_check_status(void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return qgb_host::set_error(QGB_ECUDA, "stream sync: %s", cudaGetErrorString(e));
    int status = 0;
    e = cudaMemcpyFromSymbol(&status, qgb::g_status, sizeof(int));
    if (e != cudaSuccess) return qgb_host::set_error(QGB_ECUDA, "status read: %s", cudaGetErrorString(e));
    if (status != 0) {
        const int zero = 0;
        cudaMemcpyToSymbol(qgb::g_status, &zero, sizeof(int));
        return qgb_host::set_error(QGB_ETIMEOUT, "a bounded device wait gave up (code %d)", status);
    }
    const int sweep = qgb_host::sweep_status_read_clear();
    if (sweep < 0) return qgb_host::set_error(QGB_ECUDA, "sweep status read failed");
    if (sweep != 0) return qgb_host::set_error(QGB_ETIMEOUT, "a sweep's tile-load wait gave up (code %d)", sweep);
    const int tc = qgb_host::tc_status_read_clear();
    if (tc < 0) return qgb_host::set_error(QGB_ECUDA, "tensor-core status read failed");
    if (tc != 0) return qgb_host::set_error(QGB_ETIMEOUT, "a tensor-core completion wait gave up (code %d)", tc);
    const int tcs = qgb_host::tcs_status_read_clear();
    if (tcs < 0) return qgb_host::set_error(QGB_ECUDA, "tensor-core sweep status read failed");
    if (tcs != 0) return qgb_host::set_error(QGB_ETIMEOUT, "a tensor-core sweep wait gave up (code %d)", tcs);
    const int dmb = qgb_host::dmb_status_read_clear();
    if (dmb < 0) return qgb_host::set_error(QGB_ECUDA, "density-matrix batch status read failed");
    if (dmb != 0) return qgb_host::set_error(QGB_ETIMEOUT, "a density-matrix batch wait gave up (code %d)", dmb);
    const int tj = qgb_host::traj_status_read_clear();
    if (tj < 0) return qgb_host::set_error(QGB_ECUDA, "trajectory status read failed");
    if (tj != 0) return qgb_host::set_error(QGB_EINVAL, "more than 16 jumps in one sweep of a trajectory (code %d)", tj);
    const int fu = qgb_host::fuse_status_read_clear();
    if (fu < 0) return qgb_host::set_error(QGB_ECUDA, "fusion status read failed");
    if (fu != 0) return qgb_host::set_error(QGB_EINVAL, "a fusion table entry was out of bounds (code %d)", fu);
    return QGB_OK;
}
