// ctx.h -- internal hooks of the device context (nmg.cu) used by other
// translation units of the library.
#pragma once
#include <cstddef>

#include "../../include/nmg.h"

// number of doubles in one state of the context
size_t nmg_ctx_state_len(const nmg_ctx *c);
// CUDA device the context was created on
int nmg_ctx_device(const nmg_ctx *c);
// record an error message that is a static string (no allocation) and
// return code
int nmg_ctx_fail_static(nmg_ctx *c, int code, const char *msg);
// one RK4 step u_in -> u_out on the context stream with caller-provided
// stage buffers s1, s2 (each >= state length); waits for completion.
// Applies the context's MRS limiter and exponential filter where
// nmg_rk4_step does.  Allocates nothing and never runs the autotuner (an
// untuned context uses its first compiled kernel variant).
int nmg_ctx_rk4_step_buffers(nmg_ctx *c, double t, double dt, const double *u_in,
                             double *u_out, double *s1, double *s2);
