// dropin_driver.cpp -- TEST INFRASTRUCTURE.  The reference's driver loop
// (src/main.cpp:198-216 selection of the right-hand side from the
// environment variable `parallel`, 254-300 set-up, 313-341 time loop, 355
// solution output) with the GB300 branch the integration notes add:
// parallel = 2 selects Gfunc_gpu and exprem_gpu.  The problem is read from a
// directory the test writes: problem.txt (counts, soils, boundary flux,
// initial head, end time, output times), Keff.txt (the reference's format)
// and the geometry arrays the reference's own mesh preprocessing produced
// (raw little-endian files named after the struct fields).
//
// Outputs in the directory, suffixed by the value of `parallel`:
//   g_<p>.bin         Gfunc(g, u0, user_data) at the initial state;
//   statistics_<p>.txt the reference's per-step lines (NumSteps, t,
//                      CurrentStep, CurrentKryDim), printed to 17 digits;
//   solution_<p>.bin  the tspan rows after the micro-boundary calibration
//                      the reference's save_solution applies.
// Exit status 0, or 3 when exprem returns -1 (the reference stops there).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tsr_dropin.hpp"

int Gfunc_serial(double* g, double* u, user_data_struct user_data);
int Gfunc_parallel(double* g, double* u, user_data_struct user_data);
int exprem(int (*Gfunc)(double* g, double* u, user_data_struct user_data), int N, double& t,
           double tend, double* tspan, double* tspan_solns, double* u0, user_data_struct user_data,
           exprem_options_struct options, exprem_stats_struct& stats);

static std::string g_dir;

template <typename T>
static T* load(const char* name, size_t n)
{
    std::string path = g_dir + "/" + name + ".bin";
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        std::fprintf(stderr, "missing %s\n", path.c_str());
        std::exit(2);
    }
    T* p = new T[n > 0 ? n : 1];
    size_t got = std::fread(p, sizeof(T), n, f);
    std::fclose(f);
    if (got != n) {
        std::fprintf(stderr, "short %s\n", path.c_str());
        std::exit(2);
    }
    return p;
}

static void save(const std::string& name, const double* p, size_t n)
{
    FILE* f = std::fopen((g_dir + "/" + name).c_str(), "wb");
    std::fwrite(p, sizeof(double), n, f);
    std::fclose(f);
}

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    g_dir = argv[1];
    FILE* pf = std::fopen((g_dir + "/problem.txt").c_str(), "r");
    if (!pf) return 2;
    int nv, Mn, Ne, mn, mNe, no_solns;
    double cell_area, h0, tend, bflux, A[5], B[5];
    if (std::fscanf(pf, "%d %d %d %d %d %lf %lf %lf %lf %d", &nv, &Mn, &Ne, &mn, &mNe, &cell_area, &h0,
                    &tend, &bflux, &no_solns) != 10)
        return 2;
    std::vector<double> tspan((size_t)no_solns + 1);
    tspan[0] = no_solns;
    for (int i = 1; i <= no_solns; ++i)
        if (std::fscanf(pf, "%lf", &tspan[i]) != 1) return 2;
    for (int i = 0; i < 5; ++i)
        if (std::fscanf(pf, "%lf", &A[i]) != 1) return 2;
    for (int i = 0; i < 5; ++i)
        if (std::fscanf(pf, "%lf", &B[i]) != 1) return 2;
    std::fclose(pf);

    // parallel = 0 serial, 1 OpenMP, 2 GB300 (src/main.cpp:198-213 plus the GPU branch)
    const char* pe = std::getenv("parallel");
    int parallel = pe ? std::atoi(pe) : 0;
    int (*Gfunc_type)(double* g, double* u, user_data_struct user_data);
    bool gpu = false;
    if (parallel == 0) Gfunc_type = Gfunc_serial;
    else if (parallel == 1) Gfunc_type = Gfunc_parallel;
    else if (parallel == 2) { Gfunc_type = Gfunc_gpu; gpu = true; }
    else return 2;
    const char* te = std::getenv("OMP_NUM_THREADS");
    unsigned int NUM_THREADS = te && std::atoi(te) > 0 ? (unsigned)std::atoi(te) : 1u;

    Keff_struct keff;
    if (tsr_read_effective_conductivity((g_dir + "/Keff.txt").c_str(), &keff)) return 2;
    const size_t nvNe = (size_t)nv * Ne, mNe3 = 3 * (size_t)mNe;
    macro_mesh_struct M{};
    M.no_verts = nv;
    M.no_nodes = Mn;
    M.no_elements = Ne;
    M.elements = load<int>("macro_elements", nvNe);
    M.nodes = load<double>("macro_nodes", 2 * (size_t)Mn);
    M.shape_funcs = load<double>("macro_shape_funcs", nv * nvNe);
    M.normals = load<double>("macro_normals", 2 * nvNe);
    M.boundary_edge_midpts = load<double>("macro_boundary_edge_midpts", 4 * nvNe);
    M.boundary_edge_normals = load<double>("macro_boundary_edge_normals", 4 * nvNe);
    M.boundary_edge_lens = load<double>("macro_boundary_edge_lens", 2 * nvNe);
    M.boundary_condition_edges = load<int>("macro_boundary_condition_edges", nvNe);
    M.CV_area = load<double>("macro_CV_area", (size_t)Mn);
    M.SCV_area = load<double>("macro_SCV_area", nvNe);
    M.midx = load<double>("macro_midx", nvNe);
    M.midy = load<double>("macro_midy", nvNe);
    M.centroid_elements = load<double>("macro_centroid_elements", 2 * (size_t)Ne);
    micro_mesh_struct m{};
    m.no_verts = 3;
    m.no_nodes = mn;
    m.no_elements = mNe;
    m.elements = load<int>("micro_elements", mNe3);
    m.boundary_nodes = load<int>("micro_boundary_nodes", (size_t)mn);
    m.nodes = load<double>("micro_nodes", 2 * (size_t)mn);
    m.shape_funcs = load<double>("micro_shape_funcs", 3 * mNe3);
    m.normals = load<double>("micro_normals", 2 * mNe3);
    m.boundary_edges = load<int>("micro_boundary_edges", mNe3);
    m.boundary_edge_midpts = load<double>("micro_boundary_edge_midpts", 4 * mNe3);
    m.boundary_edge_normals = load<double>("micro_boundary_edge_normals", 4 * mNe3);
    m.boundary_edge_lens = load<double>("micro_boundary_edge_lens", 2 * mNe3);
    m.centroid_elements = load<double>("micro_centroid_elements", 2 * (size_t)mNe);
    m.CV_area = load<double>("micro_CV_area", (size_t)mn);
    m.midx = load<double>("micro_midx", mNe3);
    m.midy = load<double>("micro_midy", mNe3);
    m.vectors = load<double>("micro_vectors", 2 * (size_t)mn);
    m.cell_area = cell_area;
    m.element_area = nullptr;

    soil_struct soilA{A[0], A[1], A[2], A[3], A[4], 1.0 - 1.0 / A[4]};
    soil_struct soilB{B[0], B[1], B[2], B[3], B[4], 1.0 - 1.0 / B[4]};
    exprem_options_struct exprem_options;
    tsr_set_exprem_options(&exprem_options);       // the reference's defaults
    exprem_stats_struct exprem_stats{};
    const int N = Mn + Ne * mn;
    std::vector<double> u0((size_t)N, h0);
    std::vector<double> tspan_solns((size_t)N * (no_solns + 1), 0.0);
    for (int i = 0; i < N; ++i) tspan_solns[i] = u0[i];

    user_data_struct user_data;
    user_data.macro_mesh = M;
    user_data.micro_mesh = m;
    user_data.soilA = soilA;
    user_data.soilB = soilB;
    user_data.boundary_flux = bflux;
    user_data.NUM_THREADS = NUM_THREADS;
    user_data.effective_conductivity = keff;
    user_data.model_type = 3;
    user_data.N = N;

    const std::string tag = std::to_string(parallel);
    std::vector<double> g((size_t)N);
    if (Gfunc_type(g.data(), u0.data(), user_data) != 0) return 4;
    save("g_" + tag + ".bin", g.data(), g.size());

    FILE* stats_file = std::fopen((g_dir + "/statistics_" + tag + ".txt").c_str(), "w");
    double t = 0.0;
    int flag = 0;
    while (t < tend) {
        // exprem takes one internal step and then exits
        flag = gpu ? exprem_gpu(Gfunc_type, N, t, tend, tspan.data(), tspan_solns.data(), u0.data(),
                                user_data, exprem_options, exprem_stats)
                   : exprem(Gfunc_type, N, t, tend, tspan.data(), tspan_solns.data(), u0.data(),
                            user_data, exprem_options, exprem_stats);
        if (flag == -1) break;
        std::fprintf(stats_file, "%5d %.17e %.17e %d\n", exprem_stats.NumSteps, t, exprem_stats.CurrentStep,
                     exprem_stats.CurrentKryDim);
    }
    std::fclose(stats_file);
    std::printf("N: %d   FuncEvals: %d\n", N, exprem_stats.FuncEvals);
    if (flag == -1) {
        tsr_release_all();
        return 3;
    }
    // the solution writer's calibration of the micro-boundary entries
    for (int k = 0; k <= no_solns; ++k)
        if (tsr_calibrate_micro_boundary(&user_data, nullptr, tspan_solns.data() + (size_t)k * N)) return 5;
    save("solution_" + tag + ".bin", tspan_solns.data(), tspan_solns.size());
    tsr_release_all();
    return 0;
}
