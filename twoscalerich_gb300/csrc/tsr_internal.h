// tsr_internal.h -- declarations shared by the library's host translation
// units (not part of the public C-ABI).
#ifndef TSR_INTERNAL_H
#define TSR_INTERNAL_H

#include <string>

namespace tsr {
void set_error(const std::string& msg);
const char* last_error();
// phi_1(alpha * H(1:m,1:m)); H leading dimension ldH, phi leading dimension ldP.
int phipade_host(double* phiH, const double* H, double alpha, int m, int ldH, int ldP);
// boundary condition types of the macro element edges and the boundary-edge
// mask from the tagged boundary edges (1: a node out of range)
int macro_bc_edges(int nv, int Mn, int Ne, const int* elements, int n_bedges, const int* bedges,
                   const int* macro_bc, int* bc_edges, unsigned char* is_bedge);
}  // namespace tsr

#endif
