/*
 * tsr_types.h -- the reference's hot-path data structures, redeclared with
 * identical field order and types so that a caller built against the
 * reference passes the same objects to this library unchanged.
 *
 * Replaces (field for field):
 *   macro_mesh_struct      include/macro_mesh.h:1-18
 *   micro_mesh_struct      include/micro_mesh.h:1-21
 *   Keff_struct            include/Keff.h:1-8
 *   soil_struct            include/soil.h:1-7
 *   user_data_struct       include/user_data.h:1-11
 *   exprem_options_struct  include/exprem_options.h:1-13
 *   exprem_stats_struct    include/exprem_stats.h:1-8
 *
 * Layout convention (as in the reference): component-major structure of
 * arrays, array[c * count + idx]; all reals FP64, all indices 32-bit int,
 * node indices 0-based after reading.  The unknown vector u has N =
 * no_nodes(macro) + no_elements(macro) * no_nodes(micro) entries: the macro
 * heads first, then one micro cell per macro element, cell k at
 * no_nodes(macro) + k * no_nodes(micro).
 *
 * The typedefs make the structs usable from C (the oracle, ctypes) and C++.
 * If the reference's own headers are included in the same translation unit,
 * define TSR_TYPES_FROM_REFERENCE first and this header declares nothing.
 */
#ifndef TSR_TYPES_H
#define TSR_TYPES_H

#ifndef TSR_TYPES_FROM_REFERENCE

typedef struct macro_mesh_struct {
    int    no_verts;                 /* 3 (triangles) or 4 (quadrilaterals) */
    int    no_nodes;
    int    no_elements;
    int    *elements;                /* [nv * Ne]   vertex v of element k at v*Ne+k */
    double *nodes;                   /* [2 * Mn]    x at i, y at Mn+i */
    double *shape_funcs;             /* [nv*nv*Ne]  coefficient m of vertex i at (m*nv+i)*Ne+k */
    double *normals;                 /* [2*nv*Ne]   SCV face j, component d at (2j+d)*Ne+k */
    double *boundary_edge_midpts;    /* [4*nv*Ne]   edge j, half s, component d at (4j+2s+d)*Ne+k */
    double *boundary_edge_normals;   /* [4*nv*Ne]   outward, length-weighted */
    double *boundary_edge_lens;      /* [2*nv*Ne]   edge j, half s at (2j+s)*Ne+k */
    int    *boundary_condition_edges;/* [nv*Ne]     BC type of edge j (0 = interior) */
    double *CV_area;                 /* [Mn] */
    double *SCV_area;                /* [nv*Ne] */
    double *midx;                    /* [nv*Ne]     SCV face j midpoint */
    double *midy;                    /* [nv*Ne] */
    double *centroid_elements;       /* [2*Ne] */
} macro_mesh_struct;

typedef struct micro_mesh_struct {
    int    no_nodes;
    int    no_elements;
    int    *elements;                /* [nv * mNe] */
    int    *boundary_nodes;          /* [mn] 1 on the inclusion boundary */
    double *nodes;                   /* [2 * mn] in cell coordinates */
    double *shape_funcs;             /* [nv*nv*mNe] */
    double *normals;                 /* [2*nv*mNe] */
    int    *boundary_edges;          /* [nv*mNe] 1 if edge j of element k is on the boundary */
    double *boundary_edge_midpts;    /* [4*nv*mNe] */
    double *boundary_edge_normals;   /* [4*nv*mNe] */
    double *boundary_edge_lens;      /* [2*nv*mNe] */
    double *centroid_elements;       /* [2*mNe] */
    double *CV_area;                 /* [mn] */
    double *midx;                    /* [nv*mNe] */
    double *midy;                    /* [nv*mNe] */
    double cell_area;                /* cell_width * cell_height */
    double *vectors;                 /* [2*mn] node minus cell centre */
    int    no_verts;
    double *element_area;            /* [mNe] */
} micro_mesh_struct;

typedef struct Keff_struct {
    double epsilonA;                 /* volume fraction of the connected material A */
    int    no_hvalues;
    double logr;                     /* step of the table in log10|h| (negative) */
    double logh_first;               /* log10|h| of the first row */
    double *logh_values;             /* [n] */
    double *Keff_values;             /* [4*n] component c (K11,K12,K21,K22) of row i at c*n+i */
} Keff_struct;

typedef struct soil_struct {
    double Ksat;
    double thetar;
    double thetas;
    double alpha;
    double n;
    double m;                        /* 1 - 1/n */
} soil_struct;

typedef struct user_data_struct {
    macro_mesh_struct macro_mesh;
    micro_mesh_struct micro_mesh;
    Keff_struct effective_conductivity;
    soil_struct soilA;
    soil_struct soilB;
    double boundary_flux;
    int N;
    int model_type;                  /* 1, 2 or 3 (3: inclusion flux at macro scale) */
    unsigned int NUM_THREADS;
} user_data_struct;

typedef struct exprem_options_struct {
    double AbsTol;
    double RelTol;
    int    MinKrylov;
    int    MaxKrylov;
    double MinStep;
    double MaxStep;
    int    MaxNumSteps;
    double SafetyFac;
    double MinStepDecFac;
    double MaxStepIncFac;
    double InitStep;
} exprem_options_struct;

typedef struct exprem_stats_struct {
    double  CurrentStep;
    double  CurrentTime;
    int     CurrentKryDim;
    double* CurrentSoln;
    int     NumSteps;
    int     FuncEvals;
} exprem_stats_struct;

#endif /* TSR_TYPES_FROM_REFERENCE */

/* Boundary-condition types of boundary_condition_edges (reference
 * src/main.cpp:175-178), plus the Dirichlet extension. */
#define TSR_BC_FLUX        1   /* q.n = boundary_flux (inflow per unit length) */
#define TSR_BC_NOFLUX      2
#define TSR_BC_DHDX0       3   /* dh/dx = 0 */
#define TSR_BC_DHDY0       4   /* dh/dy = 0 */
#define TSR_BC_DIRICHLET   5   /* extension: h fixed at tsr_model_ext.dirichlet_h */

/* Model settings the reference structs have no field for.  A zero-filled
 * struct (or a NULL pointer) gives the documented defaults. */
typedef struct tsr_model_ext {
    double dirichlet_h;          /* head on nodes of type-5 edges [m] */
    double specific_storage;     /* S_s added to C(h) [1/m]; <= 0 means 1e-6 */
    int    kface_mode;           /* micro face conductivity: 0 mean of the two nodes, 1 upwind */
    int    n_templates;          /* > 0: cells use per-cell micro templates (below) */
    const double* cell_scale;    /* [no_elements] inclusion scale per cell, NULL = all 1 */
    /* Batched form (uneven micro meshes; no counterpart in the reference,
     * whose user_data holds one micro mesh, include/user_data.h:4): with
     * n_templates > 0, cell k uses templates[cell_template[k]] instead of
     * user_data.micro_mesh, and the unknowns of cell k follow those of cell
     * k-1 (offsets are prefix sums of the template node counts). */
    const micro_mesh_struct* templates;   /* [n_templates] */
    const int* cell_template;             /* [no_elements] */
    const soil_struct* cell_soilB;        /* [no_elements] material B per cell, NULL = soilB */
    /* Ensemble form (no counterpart in the reference): with scenarios = S > 1
     * the macro mesh is S identical disjoint blocks (no_nodes/S nodes and
     * no_elements/S elements each, block s numbered after block s-1); the
     * unknowns are laid out scenario by scenario, [macro_s | cells_s], and
     * scenario s may carry its own material A, Keff scale and material B. */
    int scenarios;                        /* 0 or 1: one problem */
    int reserved2;
    const soil_struct* scen_soilA;        /* [S] or NULL = soilA */
    const double* scen_keff_scale;        /* [S] factor on Keff, or NULL = 1 */
    /* Learned closure (no counterpart in the reference): with cell_learned
     * non-NULL, cell k with cell_learned[k] = 1 carries one unknown, the
     * mean water content of its inclusion's interior nodes, instead of its
     * micro nodes.  The closure relaxes that water content towards the
     * water content of material B at the macro head: the exchange inflow is
     * Q = kQ (theta_B(H_c) - theta) and the rate is
     * d theta/dt = kT (theta_B(H_c) - theta), with H_c the macro head at
     * the cell centre, theta_B the retention curve of material B and
     * (kQ, kT) = closure_coef[2k], [2k+1]. */
    const int* cell_learned;              /* [no_elements] or NULL */
    const double* closure_coef;           /* [2 * no_elements] or NULL (zeros) */
} tsr_model_ext;

#endif /* TSR_TYPES_H */
