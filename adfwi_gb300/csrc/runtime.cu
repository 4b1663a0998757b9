// Error reporting and build information of the C ABI.
#include <stdarg.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#include "../../include/adfwi_gb300.h"
#include "common.cuh"

namespace adfwi {

namespace {
thread_local char g_last_error[1024] = {0};
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

void PinnedBytes::release() {
  if (ptr) {
    if (pinned)
      cudaFreeHost(ptr);
    else
      free(ptr);
  }
  ptr = nullptr;
  bytes = 0;
  pinned = false;
}

bool PinnedBytes::assign(const void* src, size_t n) {
  release();
  if (n == 0) return true;
  if (cudaMallocHost(&ptr, n) == cudaSuccess) {
    pinned = true;
  } else {
    (void)cudaGetLastError();  // no usable device here: keep a pageable copy
    ptr = malloc(n);
    if (ptr == nullptr) {
      set_error("host allocation of %zu bytes for plan tables failed", n);
      return false;
    }
  }
  memcpy(ptr, src, n);
  bytes = n;
  return true;
}

}  // namespace adfwi

extern "C" {

int adfwi_last_error(char* buf, size_t n) {
  size_t len = strlen(adfwi::g_last_error);
  if (buf != nullptr && n > 0) {
    size_t c = len < n - 1 ? len : n - 1;
    memcpy(buf, adfwi::g_last_error, c);
    buf[c] = '\0';
  }
  return (int)len;
}

const char* adfwi_version(void) { return "adfwi_gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
