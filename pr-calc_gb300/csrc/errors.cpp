// errors.cpp — per-thread last-error message.
#include "errors.h"

#include <stdarg.h>
#include <stdio.h>

#include "../../include/prc_d2z.h"

static thread_local char g_last_error[512] = "";

int prc_fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

extern "C" const char* prc_last_error(void) { return g_last_error; }
