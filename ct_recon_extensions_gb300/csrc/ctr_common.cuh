// Shared internals of libctrecon_gb300: status plumbing, launch helpers and
// the small device-math pieces every operator uses.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>

#include "ctrecon_gb300.h"

namespace ctr {

// ---- host-side status handling -------------------------------------------

// Records `msg` as this thread's last error and returns `status`.
int fail(int status, const char* fmt, ...);
// Maps the last launch error (cudaGetLastError) to a status.
int check_launch(const char* what);
// Validates the common (batch, stream) arguments and the current device.
int check_common(int batch);

inline bool bad_ptr(const void* p) { return p == nullptr; }

// ---- kernel self-checks ----------------------------------------------------
// Kernels that detect an internal inconsistency (a detector window larger
// than its shared-memory slot) set a bit here instead of trapping; the bit is
// readable with ctr_kernel_flags().
enum KernelFlag : unsigned int {
    kFlagWindowOverflow = 1u << 0,
    kFlagQueueOverflow = 1u << 1,
    kFlagWaitTimeout = 1u << 2,
    kFlagMisaligned = 1u << 3,
};
extern __device__ unsigned int g_kernel_flags;

__device__ __forceinline__ void raise_flag(unsigned int f) { atomicOr(&g_kernel_flags, f); }

// ---- launch geometry --------------------------------------------------------
constexpr int kSmCount = 152;  // GB300: 2 dies x 76 SMs

// SMs of the current device (kSmCount when the query fails).
inline int device_sms()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
        cudaGetLastError();
        return kSmCount;
    }
    return sms;
}

inline unsigned int div_up(unsigned long long a, unsigned long long b)
{
    return static_cast<unsigned int>((a + b - 1) / b);
}

// ---- programmatic dependent launch ------------------------------------------
// A kernel launched with launch_dependent may be scheduled while the kernel
// before it in the stream drains (its CTAs take the SMs the earlier grid
// frees), which hides the launch gap between consecutive operators.  Such a
// kernel calls grid_dep_wait() before it touches global memory: it returns
// once the earlier grid has completed and its writes are visible (at once
// when there is no earlier grid, or when the kernel was launched normally).
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_dependent(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                             Args&&... args)
{
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<Args&&>(args)...);
}

// ---- batched filtering (weight_filter.cu) -----------------------------------
// One item of a batched weighting + ramp-filter launch.
struct FilterJob {
    const float* in;
    float* out;
    const double* taps;   // 2*ns+1 FP64 taps of the item (RampFilterPrep layout)
    const float* weight;  // per-channel pre-weight of the item, or null
    unsigned ns, nrow;
    double ds;
};
int ramp_filter_batch_f32(const FilterJob* jobs, const int2* blocks, int n_blocks, unsigned max_ns,
                          cudaStream_t stream);
constexpr int kFilterRowsPerBlock = 4;

// ---- device math -------------------------------------------------------------
template <typename T>
struct DevMath;

template <>
struct DevMath<float> {
    static __device__ __forceinline__ float atan2_(float y, float x) { return atan2f(y, x); }
    static __device__ __forceinline__ float floor_(float x) { return floorf(x); }
    static __device__ __forceinline__ float rcp_(float x) { return __frcp_rn(x); }
    static __device__ __forceinline__ float abs_(float x) { return fabsf(x); }
};

template <>
struct DevMath<double> {
    static __device__ __forceinline__ double atan2_(double y, double x) { return atan2(y, x); }
    static __device__ __forceinline__ double floor_(double x) { return floor(x); }
    static __device__ __forceinline__ double rcp_(double x) { return 1.0 / x; }
    static __device__ __forceinline__ double abs_(double x) { return fabs(x); }
};

template <typename T>
struct Pair;
template <>
struct Pair<float> {
    using type = float2;
};
template <>
struct Pair<double> {
    using type = double2;
};

}  // namespace ctr
