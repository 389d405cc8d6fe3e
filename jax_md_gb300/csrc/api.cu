// Error reporting and library identity for the C ABI.
#include "common.cuh"

namespace jmd {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(JMD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return JMD_OK;
}

}  // namespace jmd

extern "C" {

const char* jmd_last_error(void) { return jmd::g_last_error.c_str(); }

int jmd_version(void) { return 1; }

}  // extern "C"
