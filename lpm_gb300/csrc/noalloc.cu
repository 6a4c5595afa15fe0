// noalloc.cu -- BVEVertexVelocity (FP32 compensated) with no device
// allocation at all, for callers that cannot call cudaMalloc.
//
// Who needs it: host code whose device memory is owned by another allocator
// or a fixed budget (a Kokkos memory pool, a framework's caching allocator,
// a tenant quota), where an out-of-band cudaMalloc would break the owner's
// accounting or fail; and host loops that must not stall, since cudaMalloc and
// cudaFree can synchronise the whole device.  The regular entry points keep a
// per-context scratch arena that grows with cudaMalloc; this one instead runs
// on a scratch array that is part of the loaded library.
//
// Scratch: one file-scope __device__ array of kStaticScratchBytes (64 MiB).
// Every GPU that loads this library holds it until the process exits.  Its
// device address is looked up with cudaGetSymbolAddress once per device, with
// that device current, on the first call made on that device; make that first
// call before capturing any stream.  All calls share the array and it keeps
// the previous call's contents, so calls that overlap on the GPU (different
// streams or threads at the same time) race: serialise them.  Everything the
// kernels read is written by the call first; the error flag is cleared at the
// start of every call.
#include <cmath>
#include <mutex>
#include <string>

#include "lpm_host.hpp"

namespace lpm {
namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;
constexpr size_t kFlagBytes = 256;  // error flag at the front, then the arena
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

struct DeviceScratch {
  char* base = nullptr;  // device address of g_static_scratch on this device
  int num_sms = 0;
};

std::mutex g_mutex;
DeviceScratch g_scratch[kMaxDevices];

// The host-side name g_static_scratch is not a device address; look up the
// device address for the current device (once).
DeviceScratch& scratch_for(int dev) {
  if (dev < 0 || dev >= kMaxDevices) throw Error(LPM_ERR_ARG, "device id out of range");
  std::lock_guard<std::mutex> lock(g_mutex);
  DeviceScratch& s = g_scratch[dev];
  if (!s.base) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw Error(LPM_ERR_CUDA, std::string("cudaGetSymbolAddress of the static scratch "
                                            "failed: ") + cudaGetErrorString(e));
    }
    int nsm = 0;
    LPM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    s.base = static_cast<char*>(p);
    s.num_sms = nsm;
  }
  return s;
}

// Bytes the vertex-velocity sum needs besides the chunk partials (an upper
// bound; direct_sum asks the arena for the same items).
size_t fixed_need(int64_t nverts, int64_t nfaces) {
  const int64_t tpad = (nverts + 1023) / 1024 * 1024 + 1024;  // FP32 target blocks of 1024
  const int64_t spad = (nfaces + 511) / 512 * 512 + 512;
  return 4096 + sizeof(int) * (2 * size_t(nfaces) + 2 * (size_t(nfaces) / 1024 + 2)) +
         32 * size_t(spad) + 16 * size_t(tpad) + sizeof(int) * size_t(tpad) +
         sizeof(double) * 300 + 8 * 256 + 16 * 256;
}

}  // namespace
}  // namespace lpm

namespace lpm {
int fail(int code, const char* msg);  // capi.cu
int handle_exception();               // capi.cu
}

extern "C" int lpm_bve_vertex_velocity_static(lpm_view u, lpm_view vx, int64_t nverts,
                                              lpm_view fx, const double* zeta,
                                              const double* area, const uint8_t* mask,
                                              int64_t nfaces, void* stream) {
  try {
    const int64_t kMax = (int64_t(1) << 31) - 1;
    if (nverts < 0 || nfaces < 0 || nverts > kMax || nfaces > kMax)
      return lpm::fail(LPM_ERR_ARG, "lpm_bve_vertex_velocity_static: count out of range");
    if (nverts == 0) return LPM_OK;
    if (!u.p || !vx.p || (nfaces > 0 && (!fx.p || !zeta || !area || !mask)))
      return lpm::fail(LPM_ERR_ARG, "lpm_bve_vertex_velocity_static: null pointer");
    if ((nverts > 1 && (vx.stride_i == 0 || u.stride_i == 0)) ||
        (nfaces > 1 && fx.stride_i == 0))
      return lpm::fail(LPM_ERR_ARG, "lpm_bve_vertex_velocity_static: zero row stride");
    int dev = 0;
    LPM_CUDA(cudaGetDevice(&dev));
    lpm::DeviceScratch& s = lpm::scratch_for(dev);

    const size_t cap = lpm::kStaticScratchBytes - lpm::kFlagBytes;
    const size_t base_need = lpm::fixed_need(nverts, nfaces);
    const size_t tpad = size_t((nverts + 1023) / 1024 * 1024);
    const size_t one_chunk = sizeof(double) * 3 * tpad;
    if (base_need + one_chunk + 256 > cap) {
      const std::string m = "lpm_bve_vertex_velocity_static: " + std::to_string(nverts) +
                            " targets and " + std::to_string(nfaces) + " face slots need " +
                            std::to_string(base_need + one_chunk) +
                            " bytes of scratch; the static scratch holds " +
                            std::to_string(cap) + " (use lpm_bve_vertex_velocity)";
      return lpm::fail(LPM_ERR_ARG, m.c_str());
    }

    lpm_context ctx;
    ctx.device = dev;
    ctx.stream = static_cast<cudaStream_t>(stream);
    ctx.precision = LPM_FP32C;
    ctx.num_sms = s.num_sms;
    ctx.d_err = reinterpret_cast<int*>(s.base);
    ctx.arena.base = s.base + lpm::kFlagBytes;
    ctx.arena.cap = cap;
    ctx.arena.fixed = true;
    ctx.max_part_bytes = cap - base_need - 256;
    ctx.autotune = false;  // no per-call timing runs: the default kernel shape
    LPM_CUDA(cudaMemsetAsync(ctx.d_err, 0, sizeof(int), ctx.stream));

    lpm::SumSpec spec{3, lpm::FORM_BVE, LPM_FP32C, 0.0, true, false, true};
    const lpm::SrcSpec src{lpm::to_view(fx), zeta, area, mask, nfaces};
    const lpm::TgtSeg seg{lpm::to_view(vx), nverts, lpm::to_view(u), nullptr, false};
    lpm::direct_sum(ctx, spec, src, &seg, 1);
    lpm::check_device_error(ctx);  // synchronises the stream
    ctx.arena.base = nullptr;      // not owned
    ctx.arena.cap = 0;
    return LPM_OK;
  } catch (...) {
    return lpm::handle_exception();
  }
}
