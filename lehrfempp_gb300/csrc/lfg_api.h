// Entry/exit plumbing shared by every C-ABI function: switch to the context's
// device, convert lfg::Failure / CUDA errors into status codes, remember the
// message on the context.
#pragma once

#include <new>

#include "lfg_internal.h"

#define LFG_API_BEGIN(ctx_expr)                                         \
  lfg_ctx* _lfg_ctx = (ctx_expr);                                       \
  if (!_lfg_ctx) return LFG_INVALID_ARG;                                \
  try {                                                                 \
    ::lfg::CudaCheck(cudaSetDevice(_lfg_ctx->device), "cudaSetDevice");

#define LFG_API_END                                                     \
  }                                                                     \
  catch (const ::lfg::Failure& f) {                                     \
    _lfg_ctx->last_error = f.msg;                                       \
    return f.code;                                                      \
  }                                                                     \
  catch (const std::bad_alloc&) {                                       \
    _lfg_ctx->last_error = "host allocation failed";                    \
    return LFG_OUT_OF_MEMORY;                                           \
  }                                                                     \
  _lfg_ctx->last_error.clear();                                         \
  return LFG_OK;

// Launch-check helper: counts the launch and checks the launch error.
#define LFG_LAUNCHED(ctx)                                              \
  do {                                                                  \
    ::lfg::CountLaunch(ctx);                                            \
    ::lfg::CudaCheck(cudaGetLastError(), "kernel launch");              \
  } while (0)
