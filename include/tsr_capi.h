/*
 * tsr_capi.h -- C-ABI of the GB300 two-scale Richards hot path.
 *
 * Plain pointers and sizes only.  Every call returns a status code (TSR_OK =
 * 0) and none calls exit(); tsr_last_error_message() describes the last
 * failure of the calling thread.  One process drives one GPU; a context owns
 * the device copy of the mesh geometry and every work buffer it needs, so the
 * per-call paths allocate nothing.
 *
 * Each entry point names the reference interface it replaces (paths inside
 * the TwoScaleRich source tree).  The C++ drop-ins with the reference's exact
 * signatures (Gfunc_gpu, exprem_gpu) are in tsr_dropin.hpp and are thin
 * wrappers over these functions.
 */
#ifndef TSR_CAPI_H
#define TSR_CAPI_H

#include <stddef.h>

#include "tsr_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define TSR_OK             0
#define TSR_ERR_CUDA       1   /* a CUDA runtime call failed */
#define TSR_ERR_NAN        2   /* non-finite value met in a device reduction */
#define TSR_ERR_BOUNDS     3   /* an index of the mesh data is out of range */
#define TSR_ERR_TIMEOUT    4   /* a bounded device wait ran out */
#define TSR_ERR_ARG        5   /* invalid argument or unsupported mesh */
#define TSR_ERR_ALLOC      6   /* allocation failed */
#define TSR_ERR_SINGULAR   7   /* singular Pade denominator in phipade */
#define TSR_ERR_MINSTEP    8   /* step size fell below MinStep */
#define TSR_ERR_MAXSTEPS   9   /* MaxNumSteps reached */
#define TSR_ERR_GFUNC     10   /* G evaluation reported a failure flag */
#define TSR_ERR_IO        11   /* file missing or malformed */

typedef struct tsr_ctx tsr_ctx;

int         tsr_version(void);
const char* tsr_last_error_message(void);

/* ---- host-side set-up (reference layer L0/L1, kept on the host) ------- */

/* Replaces macro_mesh_properties(const char*, macro_mesh_struct&, int*)
 * (src/macro_mesh_properties.cpp:15; prototype include/main.h:23).  Reads the
 * reference's macro mesh text format.  macro_bc[j] is the BC type of boundary
 * tag -(j+1), j = 0..4.  Returns TSR_ERR_IO where the reference returns 1. */
int tsr_macro_mesh_properties(const char* mesh_file, macro_mesh_struct* mesh,
                              const int* macro_bc);

/* Same geometry from in-memory arrays: xy[2*n_nodes] (x block then y
 * block), elems[nv*n_elems] 0-based and element-major (vertex v of element k
 * at k*nv+v), bedges[3*n_bedges] = (node a, node b, tag) 0-based nodes. */
int tsr_macro_mesh_build(int nv, int n_nodes, const double* xy, int n_elems,
                         const int* elems, int n_bedges, const int* bedges,
                         const int* macro_bc, macro_mesh_struct* mesh);

/* The same arrays as tsr_macro_mesh_build (same arguments, same host
 * struct, freed by tsr_macro_mesh_free) with the per-element geometry and
 * the control-volume areas computed on the current GPU -- the step
 * src/macro_mesh_properties.cpp:241-456 does on the host -- equal to the
 * host builder's bit for bit. */
int tsr_macro_mesh_build_device(int nv, int n_nodes, const double* xy, int n_elems,
                                const int* elems, int n_bedges, const int* bedges,
                                const int* macro_bc, macro_mesh_struct* mesh);

/* Replaces micro_mesh_properties(const char*, micro_mesh_struct&)
 * (src/micro_mesh_properties.cpp:15; include/main.h:25). */
int tsr_micro_mesh_properties(const char* mesh_file, micro_mesh_struct* mesh);

int tsr_micro_mesh_build(double cell_width, double cell_height, int nv,
                         int n_nodes, const double* xy, int n_elems,
                         const int* elems, int n_bedges, const int* bedges,
                         micro_mesh_struct* mesh);

/* Replaces read_effective_conductivity(const char*, Keff_struct&)
 * (src/read_effective_conductivity.cpp:15; include/main.h:26). */
int tsr_read_effective_conductivity(const char* Keff_file, Keff_struct* keff);

/* Replaces set_exprem_options(exprem_options_struct&)
 * (src/set_exprem_options.cpp:14; include/main.h:28). */
int tsr_set_exprem_options(exprem_options_struct* options);

void tsr_macro_mesh_free(macro_mesh_struct* mesh);
void tsr_micro_mesh_free(micro_mesh_struct* mesh);
void tsr_keff_free(Keff_struct* keff);

/* Overwrites the micro-boundary entries of u (N doubles, host) with the
 * macro interpolant, as src/save_solution.cpp:256-318 does before writing a
 * solution (the cell kernels use the interpolant there and do not evolve
 * those entries).  ext may be NULL. */
int tsr_calibrate_micro_boundary(const user_data_struct* user_data,
                                 const tsr_model_ext* ext, double* u);

/* Replaces save_solution(string, double* tspan, double* tspan_solns, int
 * no_solns, user_data_struct) (src/save_solution.cpp:14; include/main.h:33):
 * calibrates the micro-boundary entries of the no_solns + 1 rows of
 * tspan_solns in place (as above), then writes the reference's file layout
 * (the row count, then per row the time -- 0 for row 0 -- and the N values,
 * printed as %.20e).  Returns TSR_ERR_IO where the reference prints an
 * error and carries on. */
int tsr_save_solution(const char* solution_file, const double* tspan, double* tspan_solns,
                      int no_solns, const user_data_struct* user_data);

/* Keff(h) by homogenisation of the unit cell -- the table the reference
 * reads (src/read_effective_conductivity.cpp; include/Keff.h) and generates
 * with a MATLAB script it does not ship (src/main.cpp:111-112).  The macro
 * continuum is material A around the inclusion, whose triangles are
 * `inclusion` (a micro mesh, cell_width x cell_height cell, inclusion not
 * touching the cell boundary).  Solves the periodic cell problems of the
 * perforated cell (cut-face finite volumes on a resolution-wide grid,
 * conjugate gradients on the GPU to relative residual tol) and returns
 * Khom[4] (row-major: e_c . <grad chi_d + e_d>, K_A = 1) and epsA = |Y_A| /
 * |Y|.  With n_h > 0 it also fills table[5 * n_h] in the reference's
 * component-major layout: log10|h| = logh_first + r logr, then
 * K11, K12, K21, K22 = factor * K_A(10^log10|h|) * Khom (K_A the van
 * Genuchten-Mualem conductivity of soilA; factor converts its time unit). */
int tsr_keff_homogenize(const micro_mesh_struct* inclusion, double cell_width, double cell_height,
                        int resolution, double tol, const soil_struct* soilA, double factor,
                        double logh_first, double logr, int n_h, double* Khom, double* epsA,
                        double* table);

/* Replaces phipade(double*, double*, double, int, int)
 * (src/phipade.cpp:15; include/exprem.h:28): phi_1(alpha*H(1:m,1:m)) by the
 * (6,6) Pade approximant with scaling and squaring, FP64 on the host.  H has
 * leading dimension MaxKrylov+1, phiH leading dimension MaxKrylov (column
 * major).  Returns TSR_ERR_SINGULAR where the reference calls exit(). */
int tsr_phipade(double* phiH, const double* H, double alpha, int m,
                int MaxKrylov);

/* ---- device context ---------------------------------------------------- */

/* Uploads the geometry of user_data once (arrays are treated as immutable
 * afterwards, as in the reference, include/user_data.h:1-11).  stream may be
 * NULL (the context creates its own non-blocking stream).  max_krylov sizes
 * the resident Krylov basis (N x (max_krylov+1) doubles); 0 = no basis (G
 * and Jv only).  Returns NULL on failure. */
tsr_ctx* tsr_init(const user_data_struct* user_data, const tsr_model_ext* ext,
                  void* stream, int max_krylov);
void     tsr_free(tsr_ctx* ctx);
void*    tsr_stream(tsr_ctx* ctx);
int      tsr_num_unknowns(tsr_ctx* ctx);

/* g = G(u), the two-scale right-hand side.  Replaces Gfunc_serial /
 * Gfunc_parallel (int Gfunc(double* g, double* u, user_data_struct),
 * include/main.h:21-22, selected at src/main.cpp:198-213).  Host pointers;
 * copies in, computes on the GPU, copies out, synchronizes. */
int tsr_g_eval(tsr_ctx* ctx, const double* u, double* g);

/* Same on device pointers, asynchronous on the context stream. */
int tsr_g_eval_device(tsr_ctx* ctx, const double* d_u, double* d_g);

/* Finite-difference Jacobian-vector product of the EXPREM Arnoldi loop:
 * w = (G(u + eps v) - g0) * (1/eps).  Host pointers. */
int tsr_jv(tsr_ctx* ctx, const double* u, const double* g0, const double* v,
           double eps, double* w);
int tsr_jv_device(tsr_ctx* ctx, const double* d_u, const double* d_g0,
                  const double* d_v, double eps, double* d_w);

/* Total water content of state u [m^3 per m of depth]:
 * sum_i eps_A theta_A(H_i) CV_i + sum_k (|element k| / |Y|) sum_l theta_B(h_l) A_l. */
int tsr_water_content(tsr_ctx* ctx, const double* u, double* water);

/* Deterministic FP64 dot product in the library's fixed reduction order
 * (the order every Arnoldi reduction uses).  Host pointers; for tests. */
int tsr_dot(tsr_ctx* ctx, const double* x, const double* y, int n, double* out);

/* ---- EXPREM (exponential Rosenbrock-Euler, Krylov) --------------------- */

/* One accepted step, as the reference's exprem(...) (include/main.h:29-32,
 * called once per iteration at src/main.cpp:316): advances *t and u0 (host,
 * N doubles) by one accepted step no larger than tend - *t, writes every
 * tspan time it crosses into tspan_solns (row k at k*N, tspan[0] = count),
 * and updates stats.  The solver state (u, g(u), the Krylov basis) lives on
 * the GPU; u0 is copied in and out on every call.  The first call (t == 0)
 * initialises stats, as the reference leaves them uninitialised
 * (src/main.cpp:257).  Returns TSR_OK, or an error code where the reference
 * returns -1. */
int tsr_exprem_step(tsr_ctx* ctx, double* t, double tend, const double* tspan,
                    double* tspan_solns, double* u0,
                    const exprem_options_struct* options,
                    exprem_stats_struct* stats);

/* Device-resident stepping for callers that keep u on the GPU: load the
 * state once, advance, read back when needed. */
int tsr_exprem_load(tsr_ctx* ctx, const double* u_host, double t);
int tsr_exprem_advance(tsr_ctx* ctx, double tend, const double* tspan,
                       double* tspan_solns, const exprem_options_struct* options,
                       exprem_stats_struct* stats, double* t_out);
int tsr_exprem_store(tsr_ctx* ctx, double* u_host);

/* ---- checkpoint / resume (no counterpart in the reference) --------------
 * Saves the loaded state of every scenario (t, next step size, statistics,
 * status, u) to a file, and restores it into a context of the same problem;
 * stepping on continues the same trajectory (G(u) is evaluated once more
 * after the restore, so FuncEvals is one higher per scenario).  stats: one
 * per scenario.  Learned-closure contexts are not supported. */
int tsr_checkpoint_save(tsr_ctx* ctx, const char* path, const exprem_stats_struct* stats);
int tsr_checkpoint_load(tsr_ctx* ctx, const char* path, exprem_stats_struct* stats);

/* ---- ensembles (no counterpart in the reference) ------------------------
 * A context built with tsr_model_ext.scenarios = S > 1 holds S independent
 * problems whose unknowns are laid out scenario by scenario.  G, Jv and
 * water entry points above act on all of them at once.  The ensemble EXPREM
 * advances every scenario that has not reached tend by one accepted step of
 * its own size and Krylov dimension, all in the same launches; scenario s's
 * trajectory is the one it would have on its own (same reductions, same
 * order).  The state is loaded and stored with tsr_exprem_load/store (all
 * scenarios at time t). */
int tsr_num_scenarios(tsr_ctx* ctx);
/* unknowns [*first, *first + *count) of scenario s */
int tsr_scenario_range(tsr_ctx* ctx, int s, long long* first, long long* count);
/* stats, t and status are arrays of S; tspan_solns is NULL or S pointers
 * (NULL or rows of the scenario's unknowns, row k for tspan[k]).  status[s]
 * is TSR_OK or the error that stopped scenario s (it then stays where it
 * stopped); *n_running counts scenarios still short of tend. */
int tsr_ensemble_advance(tsr_ctx* ctx, double tend, const double* tspan,
                         double* const* tspan_solns,
                         const exprem_options_struct* options,
                         exprem_stats_struct* stats, double* t, int* status,
                         int* n_running);
/* Loads the state (host, N doubles) with scenario s at time t[s]; the
 * scenarios' statuses are kept (a stopped scenario stays stopped). */
int tsr_ensemble_load(tsr_ctx* ctx, const double* u_host, const double* t);
/* water content of each scenario (S doubles) */
int tsr_ensemble_water(tsr_ctx* ctx, const double* u, double* water);

/* C entry with the data of the C++ drop-in Gfunc_gpu (tsr_dropin.hpp):
 * g = G(u) for the context registered for user_data (created on first use,
 * keyed by the address of its macro element array). */
int tsr_gfunc_gpu(double* g, double* u, const user_data_struct* user_data);

/* Registers the model extension used by contexts that tsr_gfunc_gpu and
 * exprem_gpu create implicitly (call before their first use). */
int tsr_set_default_ext(const tsr_model_ext* ext, int max_krylov);

/* Releases every implicitly created context. */
void tsr_release_all(void);

/* Autotuner of the cell kernel (no counterpart in the reference): times G
 * at state u_host (host, N doubles) for every block size and shared-memory
 * budget that fits, packs cells into CTAs accordingly and keeps the fastest
 * plan.  Plans only change how cells are grouped per CTA, never the
 * results.  Outputs may be NULL. */
int tsr_autotune(tsr_ctx* ctx, const double* u_host, int reps, double* best_ms,
                 int* best_threads, int* best_budget);

/* ---- learned closure network (no reference counterpart) ----------------
 * The closure's MLP: 6 inputs -> 4 hidden layers of 64 (SiLU) -> 2 outputs,
 * BF16 weights and activations with FP32 accumulation on the tensor cores.
 * Parameters are a flat FP32 block of tsr_mlp_num_params() floats:
 * W1 [64 x 16] (input columns 6..15 zero), b1 [64], W2..W4 [64 x 64],
 * b2..b4 [64], W5 [8 x 64] (rows 2..7 zero), b5 [8]; W row-major [out][in].
 * Inputs are rows of 8 floats (6 used), outputs rows of 2 floats. */
typedef struct tsr_mlp tsr_mlp;
int      tsr_mlp_num_params(void);
tsr_mlp* tsr_mlp_create(void);
void     tsr_mlp_free(tsr_mlp* mlp);
int      tsr_mlp_set_params(tsr_mlp* mlp, const float* params);
int      tsr_mlp_get_params(tsr_mlp* mlp, float* params);
/* y = MLP(x) for n rows (host arrays); fused = 1: the fused inference kernel
 * (activations in registers), 0: the layer-by-layer training path */
int      tsr_mlp_forward(tsr_mlp* mlp, const float* x, int n, float* y, int fused);
/* mean squared error of n rows and its gradient (tsr_mlp_num_params floats) */
int      tsr_mlp_grad(tsr_mlp* mlp, const float* x, const float* y, int n, float* loss,
                      float* grad);
/* training set (n rows, copied to the device) and minibatch AdamW training:
 * `epochs` passes in a seeded random order, cosine-decayed learning rate */
int      tsr_mlp_set_data(tsr_mlp* mlp, const float* x, const float* y, long long n);
int      tsr_mlp_train(tsr_mlp* mlp, int epochs, int batch, float lr, float weight_decay,
                       unsigned long long seed, float* loss_per_epoch);
/* one AdamW step with the gradient of the last tsr_mlp_grad */
int      tsr_mlp_adamw_step(tsr_mlp* mlp, float lr, float weight_decay);

/* ---- learned closure in the two-scale system (no reference counterpart) --
 * For a context built with tsr_model_ext.cell_learned (one scenario,
 * model_type 3).  Learned cells carry one unknown (interior mean water
 * content) and use the closure coefficients; the others keep their micro
 * meshes and the plain FP64 cell kernel. */
/* new learned/micro assignment of the cells ([no_elements] 0/1); the state
 * is re-laid out on the device (micro -> learned: interior mean water
 * content; learned -> micro: the head of that content on every node) */
int tsr_closure_set_learned(tsr_ctx* ctx, const int* learned);
/* closure coefficients (kQ, kT) of every cell, 2 * no_elements doubles */
int tsr_closure_set_coef(tsr_ctx* ctx, const double* kappa);
/* current assignment, coefficients and indicator flags (each may be NULL) */
int tsr_closure_read(tsr_ctx* ctx, int* learned, double* kappa, int* flags);
/* attach the network: norm = feature means [6], feature std [6], output
 * means [2], output std [2]; zrange = accepted standardised feature range,
 * low [6] then high [6]; thr = indicator threshold on the relative change
 * of the exchange flux, qfloor = flux floor of that ratio; auto_fallback:
 * flagged cells return to their micro meshes before the next step */
int tsr_closure_attach(tsr_ctx* ctx, tsr_mlp* mlp, const double* norm, const float* zrange,
                       double thr, double qfloor, int auto_fallback);
/* a second network of the same architecture and standardisation, trained
 * from another seed (NULL detaches it): the coefficients become the mean of
 * the two networks' outputs, and a cell is also flagged when the two
 * networks' exchange inflows differ by more than thr_ens relative to
 * max(inflow, qfloor) -- their disagreement stands for the error of the
 * prediction, so a network that has not learned the closure is not used */
int tsr_closure_attach_ensemble(tsr_ctx* ctx, tsr_mlp* second, double thr_ens);
/* coefficients of the learned cells at the loaded state and the indicator */
int tsr_closure_update(tsr_ctx* ctx, int* n_flagged);
/* one accepted EXPREM step with the closure (update, fallback, step) */
int tsr_closure_advance(tsr_ctx* ctx, double tend, const double* tspan, double* tspan_solns,
                        const exprem_options_struct* options, exprem_stats_struct* stats,
                        double* t_out, int* n_fallback);
/* per-cell summary of u (NULL: the loaded state): H_c, theta, d theta/dt,
 * Q, h(theta) -- 5 doubles per cell (the training data of the network) */
int tsr_cell_summary(tsr_ctx* ctx, const double* u, double* out);

/* ---- measurement hooks (no reference counterpart) ---------------------- */

/* Enable (1) or disable (0) CUDA-event timing of the kernel classes inside
 * EXPREM steps; enabling clears earlier records.  Category 0: G and
 * finite-difference Jv evaluations; 1: the Gram-Schmidt block of an Arnoldi
 * step.  tsr_profile_read returns the summed device time (ms), the number
 * of timed launches and their summed algorithmic bytes.  The per-index
 * Arnoldi graphs carry their timing events only while profiling is on, so
 * switching it on or off makes the next steps capture them again; calling
 * it with the current setting only clears the records. */
int tsr_profile(tsr_ctx* ctx, int enable);
int tsr_profile_read(tsr_ctx* ctx, int category, double* ms, long long* count, double* bytes);

/* The cell kernel's current plan (6 ints): threads per CTA, shared-memory
 * budget, 1 if the math tables sit in shared memory (0: read through L1),
 * most cells per bundle, persistent grid, dynamic shared memory per CTA. */
int tsr_cell_plan(tsr_ctx* ctx, int* out);

/* A plan of the caller's choosing (what the autotuner sets): threads per
 * CTA (64-1024, a multiple of 32), shared-memory budget in bytes, tables in
 * shared memory (1) or read through L1 (0).  Results never depend on it. */
int tsr_set_cell_plan(tsr_ctx* ctx, int threads, int budget, int tables_smem);

/* Replay each Arnoldi step of EXPREM from a captured CUDA graph (1, the
 * default) or launch its kernels one by one (0).  Same results either way. */
int tsr_set_graphs(tsr_ctx* ctx, int enable);

/* What shaped scenario s's last accepted step (no counterpart in the
 * reference; 8 doubles): the step size proposed at its start, the size
 * taken, the accepted error estimate (weighted RMS, accept at <= 1), the
 * halvings because the Krylov space at the largest dimension was too small,
 * the rejected attempts, 1 if the next proposal was capped by
 * MaxStepIncFac, the Krylov dimension, 1 if the step was clipped to tend. */
int tsr_step_diagnostics(tsr_ctx* ctx, int s, double* out);

/* Dense-output rows of EXPREM calibrated on the device before they are
 * copied out (1) -- the micro-boundary entries then hold the macro
 * interpolant, as the reference's solution writer stores them -- or copied
 * as computed (0, the default, the reference's exprem). */
int tsr_set_calibrated_output(tsr_ctx* ctx, int enable);

/* The same calibration of a device vector of this context's layout
 * (asynchronous on the context stream). */
int tsr_calibrate_device(tsr_ctx* ctx, double* d_x);

/* Gram-Schmidt block of an Arnoldi step as one fused launch (1, the
 * default), as the j + 4 separate reduction launches (0), or fused with
 * problems of at most 16 chunks of 8,192 unknowns in one thread-block
 * cluster (2) instead of spread one warp per CTA over the GPU (1).  Same
 * results every way. */
int tsr_set_fused_gs(tsr_ctx* ctx, int enable);

/* Orthogonalisation of the Arnoldi step (the modified Gram-Schmidt loop
 * inside the reference's missing exprem, called at src/main.cpp:316-322):
 * 0 modified Gram-Schmidt, the default, in the reference's order; 1
 * classical Gram-Schmidt twice (CGS2): H(i, j) = c_i + d_i from two
 * classical passes, each dot a fixed-order reduction, four barriers and
 * 3j+10 vector passes of traffic per Arnoldi step instead of j+3 and 4j+8.
 * Its trajectories differ from modified Gram-Schmidt's by rounding and the
 * step decisions that rounding moves; they are bitwise those of the oracle
 * run with the same variant.  CGS2 takes Krylov dimensions up to 63
 * (TSR_ERR_ARG beyond). */
int tsr_set_gram_schmidt(tsr_ctx* ctx, int variant);

/* Failure paths of the bounded device waits, run on purpose (tests):
 * which = 0, the grid barrier of the fused Gram-Schmidt kernel with a CTA
 * that never arrives; 1, the tensor-core MMA barrier with nothing arriving.
 * Returns TSR_ERR_TIMEOUT (the wait ran out and raised its error flag; no
 * fault, the device stays usable). */
int tsr_wait_probe(int which);

/* Number of kernels the library has launched since it was loaded. */
unsigned long long tsr_kernel_launches(void);

/* Measured FP64 instruction throughput of the current device (independent
 * DFMA chains; ~20 ms). */
int tsr_fp64_peak(double* ops_per_s);

/* CUDA events on the context stream (slots 0..15) and the time between two
 * of them; device synchronisation; pinned host buffers for host-side I/O. */
int   tsr_mark(tsr_ctx* ctx, int slot);
int   tsr_elapsed_ms(tsr_ctx* ctx, int slot_a, int slot_b, double* ms);
int   tsr_sync(tsr_ctx* ctx);
void* tsr_pinned_alloc(size_t bytes);
void  tsr_pinned_free(void* p);

/* ---- allocation-free variant (no counterpart in the reference) ---------- */

/* *d_out = sum_i d_x[i] * d_y[i] over n doubles, in the same fixed order as
 * tsr_dot (identical bits), without a context and without allocating device
 * memory: for callers that cannot call cudaMalloc (an embedding program that
 * owns all device memory through its own pool, loops that cannot afford an
 * allocation's device-wide synchronisation).  All pointers are device
 * pointers; the call is asynchronous on `stream` (NULL: the default stream).
 * Its scratch is a fixed file-scope device array of 64 KB + 256 B that every
 * GPU loading the library keeps until exit, so n is limited to 67,108,864
 * (larger n returns TSR_ERR_ARG).  The first call on a device looks up the
 * array's device address; make it before any stream capture.  Calls share
 * the array: calls that overlap on the GPU race, so serialise them. */
int tsr_dot_device_noalloc(const double* d_x, const double* d_y, long long n,
                           double* d_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TSR_CAPI_H */
