// capi.cu -- status strings and version of the C ABI (include/sailor_gb300.h).
#include <atomic>

#include "common.cuh"

extern "C" const char *sg_status_string(int status) {
  switch (status) {
    case SG_OK: return "ok";
    case SG_ERR_INVALID_ARG: return "invalid argument (null pointer, size or alignment)";
    case SG_ERR_CUDA: return "CUDA launch failed";
    case SG_ERR_CAPACITY: return "output capacity exceeded";
    case SG_ERR_UNSUPPORTED: return "configuration not supported";
    default: return "unknown status";
  }
}

extern "C" int sg_version(void) { return 100; }

// ---------------------------------------------------------------------------
// launch-shape knobs
// ---------------------------------------------------------------------------
namespace sg {
// Process-wide: a value set by one thread is seen by launches of every
// thread after the store (relaxed atomics: each knob is independent).
static std::atomic<int> g_tune[SG_TUNE_COUNT] = {4, 128, 64, 64, 1, 0};

int tune(int knob) {
  return (knob >= 0 && knob < SG_TUNE_COUNT) ? g_tune[knob].load(std::memory_order_relaxed) : 0;
}

namespace {
constexpr int kMaxDevices = 64;
constexpr int kSmsUnknown = 128;  // only when the runtime cannot name the device (the launch fails anyway)
std::atomic<int> g_sms[kMaxDevices] = {};
}  // namespace

int num_sms() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return kSmsUnknown;
  if (dev < kMaxDevices) {
    const int c = g_sms[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return kSmsUnknown;
  if (dev < kMaxDevices) g_sms[dev].store(n, std::memory_order_relaxed);
  return n;
}
}  // namespace sg

extern "C" int sg_tune_set(int knob, int value) {
  switch (knob) {
    case SG_TUNE_FUSE_VPT:
      if (value != 1 && value != 2 && value != 4) return SG_ERR_INVALID_ARG;
      break;
    case SG_TUNE_FUSE_BLOCK:
      if (value < 32 || value > 256 || value % 32) return SG_ERR_INVALID_ARG;
      break;
    case SG_TUNE_ISECT_BLOCK:
      if (value < 32 || value > 512 || value % 32) return SG_ERR_INVALID_ARG;
      break;
    case SG_TUNE_RENDER_WARPS:
      if (value < 1 || value > 64) return SG_ERR_INVALID_ARG;
      break;
    case SG_TUNE_FUSE_TILED:
    case SG_TUNE_ISECT_WARP:
      if (value != 0 && value != 1) return SG_ERR_INVALID_ARG;
      break;
    default:
      return SG_ERR_INVALID_ARG;
  }
  sg::g_tune[knob].store(value, std::memory_order_relaxed);
  return SG_OK;
}

extern "C" int sg_tune_get(int knob) { return sg::tune(knob); }
