// oracle_adapters.cpp -- TEST INFRASTRUCTURE.  The reference's CPU entry
// points, with its exact signatures (Gfunc_serial, Gfunc_parallel and exprem,
// include/main.h:21-32), backed by the CPU oracle (oracle/tsr_oracle.c), whose
// bodies the reference does not ship.  A driver linked against these and
// against libtsr_gb300.so runs the reference's loop with parallel = 0 or 1
// on the CPU and parallel = 2 on the GPU (Gfunc_gpu / exprem_gpu), so the
// two paths can be compared through the reference's own interfaces.
//
// Compiled either with this repository's include/tsr_types.h or, beside the
// reference's own sources, with its headers (TSR_TYPES_FROM_REFERENCE); the
// structs have the same names and layouts in both.
#ifdef TSR_ADAPTERS_WITH_REFERENCE_HEADERS
#include "main.h"
#else
#include "tsr_types.h"
#endif

extern "C" {
struct oracle_problem;
oracle_problem* oracle_create(const user_data_struct* ud, const void* ext);
int oracle_g(oracle_problem* P, const double* x, double* g, int nthreads);
int oracle_exprem_step(oracle_problem* P, double* t_io, double tend, const double* tspan,
                       double* tspan_solns, double* u, const exprem_options_struct* opt,
                       exprem_stats_struct* st, int nthreads);
}

static oracle_problem* g_problem = nullptr;
static const int* g_key = nullptr;

// the oracle's problem for user_data (created on first use, keyed by the
// macro element array, which the reference never changes after set-up)
static oracle_problem* problem_for(const user_data_struct& ud)
{
    if (!g_problem || g_key != ud.macro_mesh.elements) {
        g_problem = oracle_create(&ud, nullptr);
        g_key = ud.macro_mesh.elements;
    }
    return g_problem;
}

int Gfunc_serial(double* g, double* u, user_data_struct user_data)
{
    return oracle_g(problem_for(user_data), u, g, 1);
}

int Gfunc_parallel(double* g, double* u, user_data_struct user_data)
{
    return oracle_g(problem_for(user_data), u, g, (int)user_data.NUM_THREADS);
}

int exprem(int (*Gfunc)(double* g, double* u, user_data_struct user_data), int N, double& t,
           double tend, double* tspan, double* tspan_solns, double* u0, user_data_struct user_data,
           exprem_options_struct options, exprem_stats_struct& stats)
{
    (void)N;
    const int threads = (Gfunc == Gfunc_serial) ? 1 : (int)user_data.NUM_THREADS;
    int rc = oracle_exprem_step(problem_for(user_data), &t, tend, tspan, tspan_solns, u0, &options,
                                &stats, threads);
    return rc == 0 ? 0 : -1;
}
