// Error reporting for the C ABI.
#include <string>

#include "capi_util.h"

namespace otb {

static thread_local std::string g_last_error;

otb_status set_error(otb_status code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

bool check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

}  // namespace otb

extern "C" const char* otb_last_error(void) { return otb::g_last_error.c_str(); }
extern "C" int32_t otb_version(void) { return 1; }
