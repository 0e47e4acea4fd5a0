// status.cpp -- status strings and the per-thread last-error message.
#include <stdarg.h>
#include <stdio.h>

#include "../../include/att_gb300.h"

namespace att {

static thread_local char g_last_error[512] = {0};

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

void clear_error() { g_last_error[0] = 0; }

}  // namespace att

extern "C" const char *att_last_error(void) { return att::g_last_error; }

extern "C" int att_version(void) { return 100; }

extern "C" const char *att_status_string(int status) {
    switch (status) {
        case ATT_OK: return "ok";
        case ATT_ERR_INVALID: return "invalid argument";
        case ATT_ERR_CUDA: return "CUDA error";
        case ATT_ERR_WORKSPACE: return "workspace too small";
        case ATT_ERR_UNSUPPORTED: return "unsupported combination";
        case ATT_ERR_OVERFLOW: return "int32 index overflow";
        case ATT_ERR_FORMAT: return "malformed input";
        default: return "unknown status";
    }
}
