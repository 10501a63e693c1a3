// errors.h — per-thread last-error message behind prc_last_error().
#pragma once

// Records a formatted message for the calling thread and returns `code`.
int prc_fail(int code, const char* fmt, ...)
#if defined(__GNUC__)
    __attribute__((format(printf, 2, 3)))
#endif
    ;
