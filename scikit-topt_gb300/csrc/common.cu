// Error reporting, version string and small utilities.
#include "cuda_common.cuh"

#include <string>

namespace topt {

static thread_local std::string g_last_error;

int fail(int rc, const std::string& msg) {
  g_last_error = msg;
  return rc;
}

int fail_cuda(int err, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString((cudaError_t)err);
  return TOPT_CUDA_ERROR;
}

int device_sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 152;
  return n > 0 ? n : 152;
}

}  // namespace topt

extern "C" {

const char* topt_version(void) { return "topt-gb300 0.1.0 (sm_103a)"; }

const char* topt_last_error(void) { return topt::g_last_error.c_str(); }

}  // extern "C"

extern "C" int topt_launch_count(uint64_t* out) {
  if (!out) return topt::fail(TOPT_BAD_INPUT, "launch_count: null argument");
  unsigned long long a = 0, b = 0;
  int rc = topt::launches_fem(&a);
  if (rc) return rc;
  rc = topt::launches_filter(&b);
  if (rc) return rc;
  unsigned long long c = 0;
  rc = topt::launches_design(&c);
  if (rc) return rc;
  unsigned long long d = 0;
  rc = topt::launches_heat(&d);
  if (rc) return rc;
  unsigned long long e = 0, f = 0, g = 0, k = 0;
  if ((rc = topt::launches_spmv(&e))) return rc;
  if ((rc = topt::launches_amg(&f))) return rc;
  if ((rc = topt::launches_mf(&g))) return rc;
  if ((rc = topt::launches_mf_tc(&k))) return rc;
  *out = (uint64_t)(a + b + c + d + e + f + g + k);
  return TOPT_OK;
}
