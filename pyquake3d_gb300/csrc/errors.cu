// Thread-local last-error text behind pq3d_last_error().
#include <stdarg.h>
#include <string.h>

#include "common.cuh"

namespace pq3d {

static thread_local char g_last_error[512] = "";

int set_error(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
    return code;
}

void clear_error() { g_last_error[0] = '\0'; }

}  // namespace pq3d

extern "C" const char *pq3d_last_error(void) { return pq3d::g_last_error; }
extern "C" int pq3d_version(void) { return 1; }
