// extern "C" entry points over the reference's own C++ functions, compiled
// together with the reference sources into oracle/_ref/libtsr_ref.so.  Test
// infrastructure: it lets the tests call the reference's phipade, mesh
// preprocessing, Keff reader, options and solution writer unchanged.
#include <string>

#include "macro_mesh.h"
#include "micro_mesh.h"
#include "Keff.h"
#include "soil.h"
#include "user_data.h"
#include "exprem_options.h"

int macro_mesh_properties(const char* mesh_file, macro_mesh_struct& macro_mesh, int* macro_bc);
int micro_mesh_properties(const char* mesh_file, micro_mesh_struct& micro_mesh);
int read_effective_conductivity(const char* Keff_file, Keff_struct& effective_conductivity);
int set_exprem_options(exprem_options_struct& options);
int phipade(double* phiH, double* H, double alpha, int m, int MaxKrylov);
void save_solution(std::string solution_file, double* tspan, double* tspan_solns, int no_solns,
                   user_data_struct user_data);

extern "C" {
int ref_macro_mesh_properties(const char* f, macro_mesh_struct* m, int* bc)
{
    return macro_mesh_properties(f, *m, bc);
}
int ref_micro_mesh_properties(const char* f, micro_mesh_struct* m) { return micro_mesh_properties(f, *m); }
int ref_read_effective_conductivity(const char* f, Keff_struct* k) { return read_effective_conductivity(f, *k); }
int ref_set_exprem_options(exprem_options_struct* o) { return set_exprem_options(*o); }
int ref_phipade(double* phiH, double* H, double alpha, int m, int MaxKrylov)
{
    return phipade(phiH, H, alpha, m, MaxKrylov);
}
void ref_save_solution(const char* f, double* tspan, double* solns, int no_solns, const user_data_struct* ud)
{
    save_solution(std::string(f), tspan, solns, no_solns, *ud);
}
}
