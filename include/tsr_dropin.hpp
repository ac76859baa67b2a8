// tsr_dropin.hpp -- C++ drop-ins with the reference's exact signatures.
//
// A caller built against TwoScaleRich's include/main.h selects these where
// it selects Gfunc_serial / Gfunc_parallel (src/main.cpp:198-213) and calls
// exprem_gpu where it calls exprem (src/main.cpp:316).  Both route through
// the C-ABI of tsr_capi.h; the device context for a user_data is created on
// first use (keyed by the address of its macro element array, which the
// reference never changes after set-up) and released by tsr_release_all().
#ifndef TSR_DROPIN_HPP
#define TSR_DROPIN_HPP

#include "tsr_capi.h"

// Replaces int Gfunc_serial(double* g, double* u, user_data_struct user_data)
// and Gfunc_parallel (include/main.h:21-22).  Same arguments and meaning:
// g[N] = G(u[N]) in host memory; returns 0 on success, non-zero on failure
// (a non-finite G, a CUDA error), which exprem treats as a failed step.
int Gfunc_gpu(double* g, double* u, user_data_struct user_data);

// Replaces int exprem(int (*Gfunc)(double*, double*, user_data_struct), int N,
// double& t, double tend, double* tspan, double* tspan_solns, double* u0,
// user_data_struct user_data, exprem_options_struct options,
// exprem_stats_struct& stats) (include/main.h:29-32).  Takes one accepted
// step and returns, as the reference's driver loop expects.  The Gfunc
// argument is IGNORED: the right-hand side is always the library's GPU G of
// user_data, evaluated on the device inside the Krylov loop (a host
// function pointer cannot be called there).  It is accepted only for
// signature compatibility; pass Gfunc_gpu.  The device context is the one
// registered for user_data (keyed by its macro element array, as for
// Gfunc_gpu; tsr_set_default_ext supplies model extensions before the first
// call).  Returns 0, or -1 on failure (the reference's fatal code,
// src/main.cpp:319-322).
int exprem_gpu(int (*Gfunc)(double* g, double* u, user_data_struct user_data), int N,
               double& t, double tend, double* tspan, double* tspan_solns, double* u0,
               user_data_struct user_data, exprem_options_struct options,
               exprem_stats_struct& stats);

#endif
