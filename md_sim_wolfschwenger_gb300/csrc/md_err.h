// md_err.h -- error recording shared by every translation unit of the
// library (CUDA and host-only): the message of the last failing call, per
// context and process-wide (md_last_error).
#pragma once
#include "../../include/md_gb300.h"

// Records status and message for ctx (may be NULL) and returns status.
int set_err(md_ctx* ctx, int status, const char* fmt, ...);
