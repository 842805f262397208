// Shared pieces of the C++ mirror of the reference operator API.
//
// The classes in include/ct_recon/*.h keep the names, constructors and
// calculate_on_gpu signatures of the reference's include/*.h and return bool
// as it does: true when the GPU work was launched and completed.  Each call
// synchronises the given stream (the reference synchronises the device), so the
// classes keep the reference's blocking semantics; use the C ABI in
// ctrecon_gb300.h directly for stream-ordered, non-blocking calls.
//
// calculate_on_cpu is declared for source compatibility and returns false: this
// library is the GPU implementation only (the reference's own CPU code is the
// CPU implementation).
#ifndef CT_RECON_GB300_COMMON_H_
#define CT_RECON_GB300_COMMON_H_

#include <cuda_runtime.h>

#include "ctrecon_gb300.h"

namespace ct_recon {
namespace detail {

inline bool finish(int status, cudaStream_t stream)
{
    if (status != CTR_OK) return false;
    return cudaStreamSynchronize(stream) == cudaSuccess;
}

template <typename T>
struct Precision;
template <>
struct Precision<float> {
    static constexpr bool is_double = false;
};
template <>
struct Precision<double> {
    static constexpr bool is_double = true;
};

}  // namespace detail
}  // namespace ct_recon

#endif
