// Internal helpers shared by the host and CUDA translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/topt.h"

struct topt_pattern;

namespace topt {

// Record the message of a failure for topt_last_error() and return rc.
int fail(int rc, const std::string& msg);
// Same, for CUDA errors (returns TOPT_CUDA_ERROR).
int fail_cuda(int err, const char* what);

struct topt_pattern_view {
  int64_t n_nodes, nnzb, ncontrib;
  const int32_t* rowptr;
  const int32_t* colind;
  const int64_t* cptr;
  const int32_t* contrib;
};
const topt_pattern_view view_of(const topt_pattern* p);
// kernel launches counted on the device by each CUDA translation unit
int launches_fem(unsigned long long* out);
int launches_filter(unsigned long long* out);
int launches_design(unsigned long long* out);
int launches_heat(unsigned long long* out);
int launches_spmv(unsigned long long* out);
int launches_amg(unsigned long long* out);
int launches_mf(unsigned long long* out);
int launches_mf_tc(unsigned long long* out);
int build_pattern(int64_t n_nodes, int64_t n_elem, int32_t nloc,
                  const int32_t* t, topt_pattern* P);

}  // namespace topt
