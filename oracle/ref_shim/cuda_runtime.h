// Host stand-in for the CUDA runtime (TEST INFRASTRUCTURE ONLY).
//
// It lets ros_tsdf's own tsdf_handler.cu and tsdf_container.cu compile as
// sequential host C++ for the reference-side parity harness
// (oracle/ref_harness.cpp).  The product never includes it.
//
// What each piece stands in for:
//   * __device__/__global__/__constant__/__host__ expand to nothing: kernels
//     and device functions become host functions, __constant__ parameters
//     become globals that cudaMemcpyToSymbol writes with memcpy.
//   * kernel launches: oracle/ref.py rewrites `K<<<g, b>>>(args)` in its
//     generated copy of the reference into `ref_launch(g, b, K)(args)`, which
//     runs every thread of the grid in order (block-major, then thread) on the
//     calling thread.  A child launch runs to completion before its parent
//     thread continues, a valid schedule for dynamic parallelism (the parent
//     grid is not complete before its children are).
//   * atomics are plain read-modify-writes: one thread runs at a time, so
//     every lock is free when taken and every counter is exact.
//   * device memory is host memory.  cudaMalloc adds a zeroed 16 KiB guard
//     band before and after each allocation: the reference indexes the block
//     heap with -1 for an update whose block is missing (tsdf_handler.cu:629),
//     and that write lands in the guard band instead of in other data.
//   * cudaFree of a pointer that device-side `new` returned (the reference
//     does this at tsdf_handler.cu:343-344, :706-708, :823) releases it with
//     free(): every such object is trivially destructible and libstdc++'s
//     operator new allocates with malloc.
//   * printf from reference code is dropped unless REF_VERBOSE is set in the
//     environment (the reference prints per allocated block and per deduped
//     block).
//   * events measure host wall-clock time.
#pragma once

#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <cmath>
#include <cstddef>
#include <map>
#include <memory>
#include <vector>

#define __device__
#define __host__
#define __global__
#define __constant__
#define __forceinline__ inline

struct ref_dim3 {
  unsigned x = 0, y = 0, z = 0;
};
inline ref_dim3 threadIdx, blockIdx, blockDim, gridDim;

typedef int cudaError_t;
constexpr cudaError_t cudaSuccess = 0;
typedef void* cudaStream_t;
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
  cudaMemcpyDefault = 4
};

inline const char* cudaGetErrorString(cudaError_t) { return "no error"; }
inline cudaError_t cudaPeekAtLastError() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }

namespace ref_rt {
constexpr size_t kGuard = 16384;
inline std::map<void*, void*>& allocations() {
  static std::map<void*, void*> m;
  return m;
}
inline bool verbose() {
  static int v = getenv("REF_VERBOSE") != nullptr ? 1 : 0;
  return v != 0;
}
}  // namespace ref_rt

template <class T>
inline cudaError_t cudaMalloc(T** p, size_t n) {
  char* base = static_cast<char*>(calloc(1, n + 2 * ref_rt::kGuard));
  if (base == nullptr) {
    fprintf(stderr, "ref harness: out of host memory (%zu bytes)\n", n);
    exit(3);
  }
  void* user = base + ref_rt::kGuard;
  ref_rt::allocations()[user] = base;
  *p = reinterpret_cast<T*>(user);
  return cudaSuccess;
}

inline cudaError_t cudaFree(void* p) {
  if (p == nullptr) return cudaSuccess;
  auto& m = ref_rt::allocations();
  auto it = m.find(p);
  if (it != m.end()) {
    free(it->second);
    m.erase(it);
  } else {
    free(p);
  }
  return cudaSuccess;
}

inline cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
  memmove(dst, src, n);
  return cudaSuccess;
}

template <class T>
inline cudaError_t cudaMemcpyToSymbol(T& symbol, const void* src, size_t n, size_t offset = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice) {
  memcpy(reinterpret_cast<char*>(&symbol) + offset, src, n);
  return cudaSuccess;
}

struct ref_event {
  std::chrono::steady_clock::time_point t;
};
typedef ref_event* cudaEvent_t;
inline cudaError_t cudaEventCreate(cudaEvent_t* e) {
  static std::vector<std::unique_ptr<ref_event>> pool;  // the reference never destroys its events
  pool.emplace_back(new ref_event());
  *e = pool.back().get();
  return cudaSuccess;
}
inline cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t = nullptr) {
  e->t = std::chrono::steady_clock::now();
  return cudaSuccess;
}
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) {
  *ms = std::chrono::duration<float, std::milli>(b->t - a->t).count();
  return cudaSuccess;
}

inline int atomicAdd(int* a, int v) {
  int o = *a;
  *a = o + v;
  return o;
}
inline int atomicSub(int* a, int v) {
  int o = *a;
  *a = o - v;
  return o;
}
inline int atomicCAS(int* a, int cmp, int v) {
  int o = *a;
  if (o == cmp) *a = v;
  return o;
}
inline int atomicExch(int* a, int v) {
  int o = *a;
  *a = v;
  return o;
}

// CUDA's device min(float, float) overload.
inline float min(float a, float b) { return fminf(a, b); }

// pow(float, int).  With REF_POW_FLOAT the reference's pow(x, 2) calls resolve
// to this overload in namespace tsdf (it hides ::pow there), which returns the
// correctly rounded float square x*x: the float semantics device code has.
// Without it they resolve to the C++ library's pow(float, int), which promotes
// to double: the semantics the reference's functions have when compiled as
// host code.
#ifdef REF_POW_FLOAT
namespace tsdf {
inline float pow(float x, int n) {
  if (n == 2) return x * x;
  return powf(x, (float)n);
}
}  // namespace tsdf
#endif

inline int ref_printf(const char* fmt, ...) {
  if (!ref_rt::verbose()) return 0;
  va_list ap;
  va_start(ap, fmt);
  int r = vprintf(fmt, ap);
  va_end(ap);
  return r;
}
#define printf(...) ref_printf(__VA_ARGS__)

template <class F>
struct ref_launcher {
  long long grid, block;
  F fn;
  template <class... A>
  void operator()(A... a) const {
    ref_dim3 st = threadIdx, sb = blockIdx, sbd = blockDim, sgd = gridDim;
    gridDim.x = (unsigned)grid;
    blockDim.x = (unsigned)block;
    for (long long b = 0; b < grid; ++b) {
      for (long long t = 0; t < block; ++t) {
        blockIdx.x = (unsigned)b;
        threadIdx.x = (unsigned)t;
        fn(a...);
      }
    }
    threadIdx = st;
    blockIdx = sb;
    blockDim = sbd;
    gridDim = sgd;
  }
};
template <class F>
inline ref_launcher<F> ref_launch(long long grid, long long block, F fn) {
  return ref_launcher<F>{grid, block, fn};
}
