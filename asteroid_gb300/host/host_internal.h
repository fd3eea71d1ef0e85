/* host_internal.h -- helpers shared by the C host files and the CUDA engine. */
#ifndef AST_HOST_INTERNAL_H
#define AST_HOST_INTERNAL_H

#ifdef __cplusplus
extern "C" {
#endif

/* Record a message for ast_last_error() (thread-local) and return code. */
int ast_set_error(int code, const char* fmt, ...)
#if defined(__GNUC__)
    __attribute__((format(printf, 2, 3)))
#endif
    ;

#ifdef __cplusplus
}
#endif
#endif
