// Driver for FRICO's own sources, compiled in place (oracle build only).
//
// Serves a triangle soup through a fake GMSH API (gmsh.h in ./shim) so that
// FRICO's load_from_gmsh / compute_connectivity / make_function_space build
// the mesh and RWG table, then exposes FRICO's compute_matrix,
// compute_matrix_approx, update_rhs, reorient_deltagap_edges, run_context,
// eval_fields, compute_port_values, compute_gain and bistatic_RCS_unit_Ei as
// extern "C" entry points for the tests and the golden-vector script.
// emw_ana_antenna.cpp and emw_ana_bistatic_rcs.cpp are #included (from the
// reference checkout, via the include path) because the functions needed are
// file-static there.
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "emw_ana_antenna.cpp"
#include "emw_ana_bistatic_rcs.cpp"
#include "gmsh.h"
#include "input_gmsh.h"
#include "quadratures.h"

// ------------------------------------------------------------------ fake GMSH
namespace {
struct FakeModel {
    std::vector<double> xyz;                                  // node tag t -> xyz[3*(t-1)]
    std::map<int, std::vector<std::size_t>> surf;             // tag -> node tags (3 per tri)
    std::map<int, std::vector<std::size_t>> curve;            // tag -> node tags (2 per seg)
};
FakeModel g_model;
}  // namespace

namespace gmsh {
void initialize(int, char**, bool, bool) {}
void finalize() {}
void clear() {}
void open(const std::string&) {}
namespace option { void setNumber(const std::string&, double) {} }
namespace model {
void add(const std::string&) {}
void getEntities(vectorpair& dimTags, int dim) {
    dimTags.clear();
    if (dim == 1 || dim == -1)
        for (auto& c : g_model.curve) dimTags.push_back({1, c.first});
    if (dim == 2 || dim == -1)
        for (auto& s : g_model.surf) dimTags.push_back({2, s.first});
}
void getPhysicalGroups(vectorpair& dimTags, int) { dimTags.clear(); }
void getPhysicalName(int, int, std::string& name) { name.clear(); }
void getEntitiesForPhysicalGroup(int, int, std::vector<int>& tags) { tags.clear(); }
namespace mesh {
void getNodes(std::vector<std::size_t>& nodeTags, std::vector<double>& coord, std::vector<double>& par, int, int,
              bool, bool) {
    size_t nn = g_model.xyz.size() / 3;
    nodeTags.resize(nn);
    for (size_t i = 0; i < nn; i++) nodeTags[i] = i + 1;
    coord = g_model.xyz;
    par.clear();
}
void getElementTypes(std::vector<int>& types, int dim, int tag) {
    types.clear();
    if (dim == 2 && g_model.surf.count(tag)) types.push_back(2);
    if (dim == 1 && g_model.curve.count(tag)) types.push_back(1);
}
void getElementsByType(int type, std::vector<std::size_t>& elemTags, std::vector<std::size_t>& nodeTags, int tag,
                       std::size_t, std::size_t) {
    const auto& src = type == 2 ? g_model.surf[tag] : g_model.curve[tag];
    size_t per = type == 2 ? 3 : 2;
    nodeTags = src;
    elemTags.resize(src.size() / per);
    for (size_t i = 0; i < elemTags.size(); i++) elemTags[i] = i + 1;
}
void generate(int) {}
void setOrder(int) {}
void setSize(const vectorpair&, double) {}
}  // namespace mesh
namespace occ {
int addRectangle(double, double, double, double, double, int, double) { return 1; }
int addSphere(double, double, double, double, int, double, double, double) { return 1; }
void rotate(const vectorpair&, double, double, double, double, double, double, double) {}
void synchronize() {}
}  // namespace occ
}  // namespace model
}  // namespace gmsh

// ------------------------------------------------------------------ SILO stubs (output never opened)
namespace frico {
silo::silo() : db_(nullptr) {}
silo::~silo() {}
bool silo::open(const std::string&) { return false; }
bool silo::open(const char*) { return false; }
bool silo::is_open() const { return false; }
void silo::close() {}
bool silo::add_mesh(const std::string&, const mesh&) { return false; }
bool silo::add_variable(const std::string&, const std::string&, const std::vector<double>&, var_centering) { return false; }
bool silo::add_variable(const std::string&, const std::string&, const Eigen::Matrix<double, Eigen::Dynamic, 1>&,
                        var_centering) { return false; }
bool silo::add_variable(const std::string&, const std::string&,
                        const Eigen::Matrix<std::complex<double>, Eigen::Dynamic, 1>&, var_centering) { return false; }
bool silo::add_variable(const std::string&, const std::string&, const Eigen::Matrix<double, Eigen::Dynamic, 3>&,
                        var_centering) { return false; }
bool silo::add_variable(const std::string&, const std::string&,
                        const Eigen::Matrix<std::complex<double>, Eigen::Dynamic, 3>&, var_centering) { return false; }
bool silo::add_curve(const std::string&, const std::vector<double>&, const std::vector<double>&) { return false; }
bool silo::mkdir(const std::string&) { return false; }
bool silo::chdir(const std::string&) { return false; }
std::optional<std::string> silo::curdir(void) const { return std::string("/"); }
}  // namespace frico

// ------------------------------------------------------------------ C entry points
using namespace frico;
using namespace frico::maxwell;
using cd = std::complex<double>;

namespace {
simulation* g_sim = nullptr;

void set_ctx(double freq) {
    g_sim->contexts.clear();
    freq_context c{};
    c.ctx_number = 0;
    c.frequency = freq;
    g_sim->contexts.push_back(c);
}

delta_gap make_dg(int n_itf, const int* tags, double vre, double vim) {
    delta_gap dg;
    dg.name = "feed";
    dg.phys_entity = 0;
    dg.interfaces.assign(tags, tags + n_itf);
    dg.voltage = cd(vre, vim);
    return dg;
}
}  // namespace

extern "C" {

// Returns the RWG count, or -1 multiple triangles / -2 lonely edge.
long ref_load(long nv, const double* xyz, long nt, const long* tri, const int* tags, long ncurve,
              const long* curve, const int* curve_tags, int degree, int approx, int force_sym) {
    delete g_sim;
    g_sim = new simulation();
    g_sim->cfg.degree = size_t(degree);
    g_sim->cfg.approx_matrix = approx != 0;
    g_sim->cfg.force_symmetry = force_sym != 0;
    g_model = FakeModel();
    g_model.xyz.assign(xyz, xyz + 3 * nv);
    for (long t = 0; t < nt; t++)
        for (int k = 0; k < 3; k++) g_model.surf[tags[t]].push_back(size_t(tri[3 * t + k] + 1));
    for (long c = 0; c < ncurve; c++)
        for (int k = 0; k < 2; k++) g_model.curve[curve_tags[c]].push_back(size_t(curve[2 * c + k] + 1));
    auto ok = load_from_gmsh(g_sim->msh);
    if (!ok) return ok.error().errtype == meshing_error::multiple_triangles ? -1 : -2;
    make_function_space(g_sim->msh, g_sim->bfuncs);
    return long(g_sim->bfuncs.size());
}

long ref_num_tri() { return long(g_sim->msh.triangles.size()); }

// 17 doubles per RWG, same layout as the oracle's table.
void ref_get_rwg(double* out) {
    for (size_t i = 0; i < g_sim->bfuncs.size(); i++) {
        const auto& b = g_sim->bfuncs[i];
        double* o = out + 17 * i;
        o[0] = b.Aminus; o[1] = b.Aplus; o[2] = double(b.itminus); o[3] = double(b.itplus);
        o[4] = b.pminus.x(); o[5] = b.pminus.y(); o[6] = b.pminus.z();
        o[7] = b.pplus.x(); o[8] = b.pplus.y(); o[9] = b.pplus.z();
        o[10] = b.length; o[11] = double(b.edge_index); o[12] = double(b.matrix_index);
        o[13] = b.interface ? 1.0 : 0.0; o[14] = b.interface ? double(*b.interface) : 0.0;
        o[15] = double(g_sim->msh.edges[b.edge_index].iv0);
        o[16] = double(g_sim->msh.edges[b.edge_index].iv1);
    }
}

int ref_dunavant(int degree, const double* p0, const double* p1, const double* p2, double* out) {
    auto q = dunavant(size_t(degree), point(p0[0], p0[1], p0[2]), point(p1[0], p1[1], p1[2]),
                      point(p2[0], p2[1], p2[2]));
    for (size_t k = 0; k < q.size(); k++) {
        out[4 * k] = q[k].p.x(); out[4 * k + 1] = q[k].p.y(); out[4 * k + 2] = q[k].p.z(); out[4 * k + 3] = q[k].w;
    }
    return int(q.size());
}

int ref_integrate_subtri(long t, int degree, double* out) {
    auto q = integrate_subtri(g_sim->msh, g_sim->msh.triangles[t], size_t(degree));
    for (size_t k = 0; k < q.size(); k++) {
        out[4 * k] = q[k].p.x(); out[4 * k + 1] = q[k].p.y(); out[4 * k + 2] = q[k].p.z(); out[4 * k + 3] = q[k].w;
    }
    return int(q.size());
}

void ref_compute_matrix(double freq, int approx, double* Zout) {
    set_ctx(freq);
    size_t n = g_sim->bfuncs.size();
    g_sim->contexts[0].Z = zdmatrix::Zero(long(n), long(n));
    if (approx) compute_matrix_approx(*g_sim, 0);
    else compute_matrix(*g_sim, 0);
    std::memcpy(Zout, g_sim->contexts[0].Z.data(), sizeof(cd) * n * n);
}

// 1 if the reorientation ran (signs written), 0 if FRICO leaves the signs empty.
int ref_reorient(int n_itf, const int* tags, int force, double* signs) {
    g_sim->cfg.force_reorient_deltagap = force != 0;
    g_sim->delta_gap_signs.clear();
    delta_gap dg = make_dg(n_itf, tags, 1.0, 0.0);
    reorient_deltagap_edges(*g_sim, dg, g_sim->delta_gap_signs);
    if (g_sim->delta_gap_signs.empty()) return 0;
    std::memcpy(signs, g_sim->delta_gap_signs.data(), sizeof(double) * g_sim->delta_gap_signs.size());
    return 1;
}

void ref_update_rhs_delta_gap(double freq, int n_itf, const int* tags, double vre, double vim, double* Vout) {
    set_ctx(freq);
    g_sim->contexts[0].V = zdvector::Zero(long(g_sim->bfuncs.size()));
    update_rhs(*g_sim, 0, make_dg(n_itf, tags, vre, vim));
    std::memcpy(Vout, g_sim->contexts[0].V.data(), sizeof(cd) * g_sim->bfuncs.size());
}

void ref_update_rhs_plane_wave(double freq, double theta, double phi, double ethr, double ethi, double ephr,
                               double ephi, double* Vout) {
    set_ctx(freq);
    g_sim->contexts[0].V = zdvector::Zero(long(g_sim->bfuncs.size()));
    plane_wave pw(theta, phi, cd(ethr, ethi), cd(ephr, ephi));
    update_rhs(*g_sim, 0, pw);
    std::memcpy(Vout, g_sim->contexts[0].V.data(), sizeof(cd) * g_sim->bfuncs.size());
}

static void copy_ctx_out(double* I, double* AJ, double* AdivJ, double* J) {
    auto& c = g_sim->contexts[0];
    size_t n = g_sim->bfuncs.size(), nt = g_sim->msh.triangles.size();
    if (I) std::memcpy(I, c.I.data(), sizeof(cd) * n);
    for (size_t t = 0; t < nt; t++)
        for (int k = 0; k < 3; k++) {
            if (AJ) ((cd*)AJ)[3 * t + k] = c.tri_AJ(long(t), k);
            if (J) ((cd*)J)[3 * t + k] = c.tri_J(long(t), k);
        }
    if (AdivJ) std::memcpy(AdivJ, c.tri_AdivJ.data(), sizeof(cd) * nt);
}

// run_context<delta_gap>: fill, rhs, LAPACK solve, lumping (uses the signs of the last ref_reorient).
int ref_run_context_delta_gap(double freq, int n_itf, const int* tags, double vre, double vim, double* I, double* AJ,
                              double* AdivJ, double* J) {
    set_ctx(freq);
    bool ok = run_context(*g_sim, 0, make_dg(n_itf, tags, vre, vim));
    copy_ctx_out(I, AJ, AdivJ, J);
    return ok ? 0 : -1;
}

int ref_run_context_plane_wave(double freq, double theta, double phi, double ethr, double ethi, double ephr,
                               double ephi, double* I, double* AJ, double* AdivJ, double* J) {
    set_ctx(freq);
    plane_wave pw(theta, phi, cd(ethr, ethi), cd(ephr, ephi));
    bool ok = run_context(*g_sim, 0, pw);
    copy_ctx_out(I, AJ, AdivJ, J);
    return ok ? 0 : -1;
}

void ref_eval_fields(long npts, const double* P, double* E, double* H) {
    for (long i = 0; i < npts; i++) {
        auto [e, h] = eval_fields(*g_sim, 0, point(P[3 * i], P[3 * i + 1], P[3 * i + 2]));
        for (int k = 0; k < 3; k++) {
            ((cd*)E)[3 * i + k] = e(k);
            ((cd*)H)[3 * i + k] = h(k);
        }
    }
}

// compute_port_values: out = {I.re, I.im, P.re, P.im, Z.re, Z.im, gamma.re, gamma.im, swr}
void ref_port_values(int n_itf, const int* tags, double vre, double vim, double Z0, double* out) {
    antenna_analysis anta;
    anta.dgap = make_dg(n_itf, tags, vre, vim);
    anta.rdiag_dist = 10;
    anta.antdata.resize(1);
    g_sim->cfg.Z0 = Z0;
    compute_port_values(*g_sim, 0, anta);
    const auto& p = anta.antdata[0].port;
    double v[9] = {p.current.real(), p.current.imag(), p.power.real(), p.power.imag(), p.impedance.real(),
                   p.impedance.imag(), p.gamma.real(), p.gamma.imag(), p.swr};
    std::memcpy(out, v, sizeof v);
}

void ref_gain(double pwr, double R, int plane, double* out) {
    std::vector<double> G;
    compute_gain(*g_sim, 0, pwr, R, plane == 0 ? gain_plane::xy : plane == 1 ? gain_plane::yz : gain_plane::xz, G);
    std::memcpy(out, G.data(), sizeof(double) * G.size());
}

// The 359-angle loop of the bistatic postpro_context (file output omitted):
// rows {VV_theta, HH_theta, VV_phi, HH_phi}.
void ref_bistatic(double R, double* out) {
    for (int i = 0; i < 359; i++) {
        double deg2rad = M_PI / 180.0;
        auto p_theta = sph2rect(R, deg2rad * i, 0.0);
        auto [Es_theta, Hs_theta] = eval_fields(*g_sim, 0, p_theta);
        auto [VV_theta, HH_theta] = bistatic_RCS_unit_Ei(Es_theta, deg2rad * i, 0.0, R);
        auto p_phi = sph2rect(R, 0.0, deg2rad * i);
        auto [Es_phi, Hs_phi] = eval_fields(*g_sim, 0, p_phi);
        auto [VV_phi, HH_phi] = bistatic_RCS_unit_Ei(Es_phi, 0.0, deg2rad * i, R);
        out[4 * i] = VV_theta; out[4 * i + 1] = HH_theta; out[4 * i + 2] = VV_phi; out[4 * i + 3] = HH_phi;
    }
}

}  // extern "C"
