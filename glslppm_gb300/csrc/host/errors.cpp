// Thread-local last-error message of the C ABI.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "scene_internal.h"

namespace {
thread_local std::string g_last_error;
}

namespace sppm {

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

int fail(int status, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

float sqrt_f32(float x) { return std::sqrt(x); }

}  // namespace sppm

extern "C" size_t sppm_last_error(char* buf, size_t buf_size) {
    if (buf && buf_size > 0) {
        const size_t n = g_last_error.size() < buf_size - 1 ? g_last_error.size() : buf_size - 1;
        memcpy(buf, g_last_error.data(), n);
        buf[n] = '\0';
    }
    return g_last_error.size();
}

extern "C" uint32_t sppm_abi_version(void) { return SPPM_ABI_VERSION; }
