// Policy backward for callers that cannot allocate device memory.
//
// racer_policy_backward needs a few megabytes of scratch for the split-K
// partial sums of its weight-gradient GEMMs; the policy object allocates it
// with cudaMalloc when it is created. Some hosts cannot do that: their device
// memory belongs to another runtime's allocator (a Mojo/MAX host whose
// DeviceContext owns every buffer, or an application that pools all device
// memory up front under a fixed budget), so a library that calls cudaMalloc
// behind their back breaks their accounting or fails outright.
// racer_policy_backward_noalloc serves them: the caller passes every input
// and output, and the scratch is the file-scope device array below, part of
// the library image itself.
//
// Limits and sharing:
//  - The array holds STATIC_SCRATCH_FLOATS floats (4.75 MiB). Every GPU that
//    loads the library holds its own copy until the process exits.
//  - Every call on a device uses the same array, and it keeps whatever the
//    previous call wrote. Calls whose kernels overlap on the GPU (two streams,
//    or two host threads) race on it; serialise them on one stream.
//  - Nothing in it needs to start at zero: each split of the GEMMs writes its
//    whole partial tile before the reduction reads it.
//  - The first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
//  - That address is kept for the life of the process. A cudaDeviceReset
//    unloads the library's device image, and the array may come back at
//    another address: do not use this entry point on a device after resetting
//    it.
//  - The split plan of the GEMMs (SPLIT_CTAS in kernels.h) is the same for
//    every size and device and bounds the partials by BACKWARD_SCRATCH_FLOATS,
//    which the array holds (checked at compile time); the size check in the
//    entry point restates that bound for the sizes of each call.
#include <mutex>
#include <string>
#include <vector>

#include "../../include/racer.h"
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr size_t STATIC_SCRATCH_FLOATS = (size_t)2 * 152 * 64 * 64;
static_assert(STATIC_SCRATCH_FLOATS >= racer::BACKWARD_SCRATCH_FLOATS,
              "the static scratch must hold every split-K plan of launch_backward");

static __device__ __align__(256) float g_static_scratch[STATIC_SCRATCH_FLOATS];

std::mutex g_lock;
std::vector<float*> g_address;  // per device; the host-side name of the array is not a device address

int static_scratch(float** out) {
  int dev = 0;
  RACER_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> guard(g_lock);
  if ((int)g_address.size() <= dev) g_address.resize(dev + 1, nullptr);
  if (!g_address[dev]) {
    void* p = nullptr;
    RACER_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
    g_address[dev] = static_cast<float*>(p);
  }
  *out = g_address[dev];
  return 0;
}

}  // namespace

extern "C" int racer_policy_backward_noalloc(int beams, const float* theta, const float* x, int cols,
                                             const float* h1, const float* h2, const float* d3, float* d2, float* d1,
                                             float* grad, void* stream) {
  using racer_host::set_error;
  if (beams < 2 || cols < 1 || !theta || !x || !h1 || !h2 || !d3 || !d2 || !d1 || !grad) {
    set_error("racer_policy_backward_noalloc: bad argument");
    return 1;
  }
  const int in = beams + 5;
  size_t need = racer::backward_scratch_needed(in, cols);
  if (need > STATIC_SCRATCH_FLOATS) {
    set_error("racer_policy_backward_noalloc: needs " + std::to_string(need) + " scratch floats, the static array holds " +
              std::to_string(STATIC_SCRATCH_FLOATS));
    return 1;
  }
  float* scratch = nullptr;
  if (int rc = static_scratch(&scratch)) return rc;
  racer::launch_backward(in, theta, x, cols, h1, h2, d3, d2, d1, grad, scratch, (cudaStream_t)stream);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) {
    set_error(std::string("racer_policy_backward_noalloc: ") + cudaGetErrorString(err));
    return 2;
  }
  return 0;
}
