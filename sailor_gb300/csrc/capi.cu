// capi.cu -- status strings and version of the C ABI (include/sailor_gb300.h).
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
