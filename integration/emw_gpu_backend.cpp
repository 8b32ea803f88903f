// emw_gpu_backend.cpp -- FRICO-side adapter onto libfrico_gpu's C-ABI.
//
// A FRICO maintainer adds this file as src/emw_gpu_backend.cpp (built with
// -DFRICO_WITH_GB300, linked with -lfrico_gpu). It keeps FRICO's own types
// (simulation, freq_context, Eigen containers) on its side of the boundary and
// passes plain arrays to include/frico_gpu.h. tests/test_integration_adapter.py
// compiles this file against FRICO's headers.
#include "frico_gpu.h"
#include "emw_solver.h"
#include "emw_postpro_common.h"

namespace frico::maxwell {

struct gpu_backend {
    frico_gpu_ctx* ctx = nullptr;
    bool mesh_loaded = false;
};
static gpu_backend g_gpu;

static void check(int rc) {
    if (rc != FRICO_GPU_OK)
        throw std::runtime_error(frico_gpu_last_error(g_gpu.ctx));
}

// Called once after init_simulation (src/emw_solver.cpp:418-458).
void gpu_attach(simulation& sim, bool mixed_precision) {
    frico_gpu_options o{};
    o.degree = int(sim.cfg.degree);            // config::degree          (-k)
    o.approx = sim.cfg.approx_matrix;          // config::approx_matrix   (-A)
    o.force_symmetry = sim.cfg.force_symmetry; // config::force_symmetry  (-S)
    o.precision = mixed_precision ? FRICO_PREC_MIXED : FRICO_PREC_FP64;
    o.Z0 = sim.cfg.Z0;                         // config::Z0              (-Z)
    check(frico_gpu_ctx_create(&g_gpu.ctx, 0, &o));

    // mesh + RWG table exactly as make_function_space built them
    std::vector<double> xyz;  std::vector<int64_t> tri;  std::vector<frico_rwg> rwg;
    for (auto& v : sim.msh.vertices) { xyz.push_back(v.x()); xyz.push_back(v.y()); xyz.push_back(v.z()); }
    for (auto& t : sim.msh.triangles) { tri.push_back(t.iv0); tri.push_back(t.iv1); tri.push_back(t.iv2); }
    for (auto& b : sim.bfuncs) {
        frico_rwg r{};
        r.Aminus = b.Aminus; r.Aplus = b.Aplus; r.itminus = b.itminus; r.itplus = b.itplus;
        r.pminus[0] = b.pminus.x(); r.pminus[1] = b.pminus.y(); r.pminus[2] = b.pminus.z();
        r.pplus[0] = b.pplus.x();   r.pplus[1] = b.pplus.y();   r.pplus[2] = b.pplus.z();
        r.length = b.length; r.edge_index = b.edge_index; r.matrix_index = b.matrix_index;
        r.has_interface = bool(b.interface); r.interface_tag = b.interface ? *b.interface : 0;
        rwg.push_back(r);
    }
    check(frico_gpu_set_mesh(g_gpu.ctx, sim.msh.vertices.size(), xyz.data(), sim.msh.triangles.size(),
                             tri.data(), rwg.size(), rwg.data()));
}

// compute_matrix / compute_matrix_approx (src/emw_solver.h:85-86). Z stays on
// the GPU; pass context.Z.data() instead of nullptr only when it is dumped (-d).
void compute_matrix_gpu(simulation& sim, size_t ctx_number) {
    check(frico_gpu_fill(g_gpu.ctx, sim.contexts[ctx_number].frequency, nullptr, 0));
}

// update_rhs(delta_gap) (src/emw_solver.h:87)
void update_rhs_gpu(simulation& sim, size_t ctx_number, const delta_gap& dg) {
    check(frico_gpu_set_nrhs(g_gpu.ctx, 1));
    frico_c128 v0{dg.voltage.real(), dg.voltage.imag()};
    const double* signs = sim.delta_gap_signs.empty() ? nullptr : sim.delta_gap_signs.data();
    check(frico_gpu_rhs_delta_gap(g_gpu.ctx, sim.contexts[ctx_number].frequency, 0, int(dg.interfaces.size()),
                                  dg.interfaces.data(), v0, signs));
}

// run_context (src/emw_solver.h:92-167) for the delta gap: fill, rhs, solve,
// lumping; I, tri_AJ, tri_AdivJ, tri_J come back into the Eigen containers.
bool run_context_gpu(simulation& sim, size_t ctx_number, const delta_gap& dg) {
    auto& c = sim.contexts[ctx_number];
    const auto n = sim.bfuncs.size(), nt = sim.msh.triangles.size();
    compute_matrix_gpu(sim, ctx_number);
    update_rhs_gpu(sim, ctx_number, dg);
    c.I = zdvector::Zero(n);
    int32_t info = 0;
    int rc = frico_gpu_solve(g_gpu.ctx, reinterpret_cast<frico_c128*>(c.I.data()), n, &info);
    if (rc == FRICO_GPU_ESINGULAR) { std::println(stderr, "ZGETRF singular matrix"); return false; }
    check(rc);
    std::vector<frico_c128> aj(3 * nt), adj(nt), j(3 * nt);
    check(frico_gpu_lump_currents(g_gpu.ctx, 0, aj.data(), adj.data(), j.data()));
    c.tri_AJ = zdfield::Zero(nt, 3); c.tri_AdivJ = zdvector::Zero(nt); c.tri_J = zdfield::Zero(nt, 3);
    for (size_t t = 0; t < nt; t++) {
        for (int k = 0; k < 3; k++) {
            c.tri_AJ(t, k) = {aj[3 * t + k].re, aj[3 * t + k].im};
            c.tri_J(t, k) = {j[3 * t + k].re, j[3 * t + k].im};
        }
        c.tri_AdivJ(t) = {adj[t].re, adj[t].im};
    }
    return true;
}

// solve_general / solve_symmetric (src/lapack_wrappers.h:10-19) on a Z that FRICO
// assembled itself (with the mesh attached by gpu_attach): upload A, solve on the
// GPU, download x. The call site in run_context (src/emw_solver.h:124-132) passes
// the context's frequency, which later field evaluations use; with -A / -S only
// A's upper triangle is read, as zsytrf with uplo = 'U' reads it.
bool solve_general_gpu(double frequency, zdmatrix& A, const zdvector& b, zdvector& x) {
    check(frico_gpu_set_matrix(g_gpu.ctx, frequency, reinterpret_cast<const frico_c128*>(A.data()), A.rows()));
    check(frico_gpu_set_rhs(g_gpu.ctx, 1, reinterpret_cast<const frico_c128*>(b.data()), b.rows()));
    x = zdvector::Zero(b.rows());
    int32_t info = 0;
    int rc = frico_gpu_solve(g_gpu.ctx, reinterpret_cast<frico_c128*>(x.data()), x.rows(), &info);
    if (rc == FRICO_GPU_ESINGULAR) { std::println(stderr, "ZGETRF singular matrix"); return false; }
    check(rc);
    return true;
}

// eval_fields (src/emw_postpro_common.h:33-34): the point-set overload.
void eval_fields_gpu(const simulation&, size_t, const mesh& smp, zdfield& E, zdfield& H) {
    const auto np = smp.vertices.size();
    std::vector<double> P;
    for (auto& v : smp.vertices) { P.push_back(v.x()); P.push_back(v.y()); P.push_back(v.z()); }
    std::vector<frico_c128> e(3 * np), h(3 * np);
    check(frico_gpu_eval_fields(g_gpu.ctx, 0, np, P.data(), e.data(), h.data()));
    E = zdfield::Zero(np, 3); H = zdfield::Zero(np, 3);
    for (size_t i = 0; i < np; i++)
        for (int k = 0; k < 3; k++) {
            E(i, k) = {e[3 * i + k].re, e[3 * i + k].im};
            H(i, k) = {h[3 * i + k].re, h[3 * i + k].im};
        }
}

}  // namespace frico::maxwell
