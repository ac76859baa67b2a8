// tsr_dropin.cpp -- the reference-signature C++ entry points (tsr_dropin.hpp).
#include <cstdio>

#include "../../include/tsr_dropin.hpp"
#include "tsr_internal.h"

namespace tsr {
tsr_ctx* registry_get(const user_data_struct* ud, int* rc);
}

int Gfunc_gpu(double* g, double* u, user_data_struct user_data)
{
    return tsr_gfunc_gpu(g, u, &user_data);
}

int exprem_gpu(int (*Gfunc)(double* g, double* u, user_data_struct user_data), int N, double& t,
               double tend, double* tspan, double* tspan_solns, double* u0,
               user_data_struct user_data, exprem_options_struct options,
               exprem_stats_struct& stats)
{
    (void)Gfunc;
    int rc = 0;
    tsr_ctx* c = tsr::registry_get(&user_data, &rc);
    if (!c) {
        std::fprintf(stderr, "exprem_gpu: %s\n", tsr::last_error());
        return -1;
    }
    if (tsr_num_unknowns(c) != N) {
        std::fprintf(stderr, "exprem_gpu: N does not match user_data\n");
        return -1;
    }
    rc = tsr_exprem_step(c, &t, tend, tspan, tspan_solns, u0, &options, &stats);
    if (rc != TSR_OK) {
        std::fprintf(stderr, "exprem_gpu: %s\n", tsr::last_error());
        return -1;
    }
    return 0;
}
