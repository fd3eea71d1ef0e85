/* errors.c -- status codes and the per-thread error message (host, C).
 *
 * The reference reports a failure by printing it and calling exit() (cuda_errors.h:4-14,
 * read_data.c:31-51).  A library cannot exit its caller, so every entry point returns an
 * AST_E_* status and keeps the message here for ast_last_error(). */
#include <stdarg.h>
#include <stdio.h>
#include "asteroid_gb300.h"
#include "host_internal.h"

static _Thread_local char g_msg[512];

int ast_set_error(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    return code;
}

const char* ast_last_error(void) { return g_msg; }

const char* ast_version(void) { return "asteroid_gb300 0.1 (sm_103a)"; }
