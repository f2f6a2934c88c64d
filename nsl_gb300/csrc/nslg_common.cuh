// Common definitions for the NSL fermion-matrix GPU library (libnslgpu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "nsl_gb300.h"

namespace nslg {

// ---------------------------------------------------------------------------------------------------------------
// Error reporting: every entry point returns an nslg_status; the message of the last failure on this host thread
// is kept for nslg_last_error().
// ---------------------------------------------------------------------------------------------------------------
void set_error(const std::string &msg);

struct Status {
    int code = NSLG_OK;
};

#define NSLG_CUDA(call)                                                                                   \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            ::nslg::set_error(std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + __FILE__ + ":" + \
                              std::to_string(__LINE__) + ")");                                            \
            return NSLG_ERR_CUDA;                                                                         \
        }                                                                                                 \
    } while (0)

#define NSLG_TRY(...)                   \
    do {                                \
        int s_ = (__VA_ARGS__);         \
        if (s_ != NSLG_OK) return s_;   \
    } while (0)

#define NSLG_REQUIRE(cond, code, msg)   \
    do {                                \
        if (!(cond)) {                  \
            ::nslg::set_error(msg);     \
            return (code);              \
        }                               \
    } while (0)

// ---------------------------------------------------------------------------------------------------------------
// Complex helpers (interleaved re/im, the layout of complex128 NSL::Tensor / torch storage)
// ---------------------------------------------------------------------------------------------------------------
template <typename T> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };
template <typename T> using cplx_t = typename Cplx<T>::type;

template <typename C> __host__ __device__ __forceinline__ C cmake(double re, double im) {
    C c;
    c.x = re;
    c.y = im;
    return c;
}
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
    C c;
    c.x = a.x * b.x - a.y * b.y;
    c.y = a.x * b.y + a.y * b.x;
    return c;
}
// conj(a) * b
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b) {
    C c;
    c.x = a.x * b.x + a.y * b.y;
    c.y = a.x * b.y - a.y * b.x;
    return c;
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Number of SMs of the current device (cached per device).
int num_sms();

// Process-wide count of kernels this library launched (graph replays count every kernel node). Launches recorded
// into a graph under stream capture are counted when the graph is replayed, not when captured.
void note_launch(cudaStream_t st, uint64_t n = 1);
uint64_t launches();

}  // namespace nslg
