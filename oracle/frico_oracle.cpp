// CPU oracle for the FRICO Method-of-Moments hot path.
//
// TEST INFRASTRUCTURE ONLY. This file restates FRICO's own CPU algorithms in
// plain C++ (std::complex<double>, OpenMP), loop for loop and expression for
// expression, so that the GPU library can be checked against it and timed
// beside it. Only the tests, the smoke check and the CPU-baseline leg of the
// benchmark load it; the product library never does.
//
// Restated functions (FRICO file:line):
//   area_triangle_kahan, dunavant, integrate, integrate_subtri
//                                  src/quadratures.cpp:41-57, 321-372, 2678-2702
//   barycenter, measure            src/geom_mesh.cpp:39-78
//   load_from_gmsh connectivity    src/input_gmsh.cpp:129-140, 216-322, 335-394
//   make_function_space            src/rwg_basis.cpp:27-68
//   compute_matrix                 src/emw_solver.cpp:45-142
//   compute_matrix_approx          src/emw_solver.cpp:144-220
//   reorient_deltagap_edges        src/emw_solver.cpp:222-350
//   update_rhs(delta_gap)          src/emw_solver.cpp:352-378
//   update_rhs(plane_wave)         src/emw_solver.cpp:380-416, src/sources.h:34-75
//   run_context current lumping    src/emw_solver.h:137-164
//   eval_fields                    src/emw_postpro_common.cpp:31-90
//   compute_gain / port values     src/emw_ana_antenna.cpp:33-105
//   bistatic_RCS_unit_Ei           src/emw_ana_bistatic_rcs.cpp:62-82
// The LAPACK step (zgetrf/zgetrs, zsytrf/zsytrs) is called from Python through
// scipy's LAPACK, the same routines FRICO links (src/lapack_wrappers.cpp).
#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <list>
#include <stdexcept>
#include <vector>

#include "../frico_gb300/csrc/dunavant_rules.h"

#define MU0 1.256637061435917e-06
#define EPS0 8.8541878188e-12

namespace {

using cd = std::complex<double>;

struct vec3 {
    double x, y, z;
};
inline vec3 operator+(vec3 a, vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(vec3 a, vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(vec3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline vec3 operator*(double s, vec3 a) { return a * s; }
inline vec3 operator/(vec3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm(vec3 v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }

struct cvec3 {
    cd x, y, z;
};

struct qpoint {
    vec3 p;
    double w;
};

struct Tri {
    int64_t v[3];
};

struct Bf {
    double Aminus, Aplus;
    int64_t itminus, itplus;
    vec3 pminus, pplus;
    double length;
    int64_t edge_index, matrix_index;
    int has_itf;
    int itf;
    vec3 rho_minus(vec3 r) const { return r - pminus; }
    vec3 rho_plus(vec3 r) const { return r - pplus; }
    vec3 eval_minus(vec3 r) const { return (-length * rho_minus(r)) / (2.0 * Aminus); }
    vec3 eval_plus(vec3 r) const { return (length * rho_plus(r)) / (2.0 * Aplus); }
    double div_minus() const { return -length / Aminus; }
    double div_plus() const { return length / Aplus; }
};

double area_triangle_kahan(vec3 p0, vec3 p1, vec3 p2) {
    const double l10 = norm(p1 - p0);
    const double l20 = norm(p2 - p0);
    const double l21 = norm(p2 - p1);
    std::array<double, 3> length{l10, l20, l21};
    std::sort(length.begin(), length.end());
    const double a = length[2], b = length[1], c = length[0];
    return 0.25 * std::sqrt((a + (b + c)) * (c - (a - b)) * (c + (a - b)) * (a + (b - c)));
}

std::vector<qpoint> dunavant(size_t degree, vec3 p0, vec3 p1, vec3 p2) {
    if (degree > 20) throw std::invalid_argument("Dunavant quadrature: degree too high");
    size_t rule = degree == 0 ? 0 : degree - 1;
    double area = area_triangle_kahan(p0, p1, p2);
    std::vector<qpoint> ret;
    ret.reserve(frico_tables::kDunavantPoints[rule]);
    for (int e = frico_tables::kDunavantFirst[rule]; e < frico_tables::kDunavantFirst[rule + 1]; e++) {
        const double* dp = frico_tables::kDunavantOrbits[e];
        int perms = int(dp[0]);
        double l0 = dp[1], l1 = dp[2], l2 = dp[3], w = dp[4];
        switch (perms) {
            case 1:
                ret.push_back({p0 * l0 + p1 * l1 + p2 * l2, w * area});
                break;
            case 3:
                ret.push_back({p0 * l0 + p1 * l1 + p2 * l2, w * area});
                ret.push_back({p0 * l1 + p1 * l2 + p2 * l0, w * area});
                ret.push_back({p0 * l1 + p1 * l0 + p2 * l2, w * area});
                break;
            case 6:
                ret.push_back({p0 * l0 + p1 * l1 + p2 * l2, w * area});
                ret.push_back({p0 * l0 + p1 * l2 + p2 * l1, w * area});
                ret.push_back({p0 * l1 + p1 * l0 + p2 * l2, w * area});
                ret.push_back({p0 * l1 + p1 * l2 + p2 * l0, w * area});
                ret.push_back({p0 * l2 + p1 * l0 + p2 * l1, w * area});
                ret.push_back({p0 * l2 + p1 * l1 + p2 * l0, w * area});
                break;
        }
    }
    return ret;
}

struct Mesh {
    std::vector<vec3> verts;
    std::vector<Tri> tris;
    std::vector<int> tri_tags;
    std::vector<std::pair<int64_t, int64_t>> edges;
    std::vector<Bf> bfs;

    vec3 bar(int64_t t) const {
        return (verts[tris[t].v[0]] + verts[tris[t].v[1]] + verts[tris[t].v[2]]) / 3.0;
    }
    double area(int64_t t) const {
        vec3 e0 = verts[tris[t].v[1]] - verts[tris[t].v[0]];
        vec3 e1 = verts[tris[t].v[2]] - verts[tris[t].v[1]];
        return 0.5 * norm(cross(e0, e1));
    }
    std::vector<qpoint> integrate(int64_t t, size_t deg) const {
        return dunavant(deg, verts[tris[t].v[0]], verts[tris[t].v[1]], verts[tris[t].v[2]]);
    }
    std::vector<qpoint> integrate_subtri(int64_t t, size_t deg) const {
        vec3 p0 = verts[tris[t].v[0]], p1 = verts[tris[t].v[1]], p2 = verts[tris[t].v[2]];
        vec3 b = bar(t);
        auto ret = dunavant(deg, p0, p1, b);
        auto q = dunavant(deg, p1, p2, b);
        ret.insert(ret.end(), q.begin(), q.end());
        q = dunavant(deg, p2, p0, b);
        ret.insert(ret.end(), q.begin(), q.end());
        return ret;
    }
};

struct State {
    Mesh msh;
    size_t degree = 1;
    int h_physical = 0;
    // per-frequency results
    double freq = 0;
    std::vector<cd> tri_AJ, tri_AdivJ, tri_J;
};

}  // namespace

extern "C" {

void* oracle_create() { return new State(); }
void oracle_destroy(void* s) { delete (State*)s; }
void oracle_set_degree(void* s, int degree, int h_physical) {
    ((State*)s)->degree = size_t(degree);
    ((State*)s)->h_physical = h_physical;
}

// load_from_gmsh (compaction, sorted edges, connectivity) + make_function_space.
// Returns the RWG count, or -1 (multiple triangles) / -2 (lonely curve edge).
int64_t oracle_set_mesh(void* sp, int64_t nv, const double* xyz, int64_t nt, const int64_t* tri,
                        const int32_t* tags, int64_t ncurve, const int64_t* curve, const int32_t* curve_tags,
                        int edge_xy) {
    State* s = (State*)sp;
    Mesh& m = s->msh;
    m = Mesh();
    // compaction: used vertices renumbered in increasing order
    std::vector<int64_t> used(nv, -1);
    for (int64_t i = 0; i < 3 * nt; i++) used[tri[i]] = 1;
    int64_t ci = 0;
    for (auto& u : used)
        if (u >= 0) u = ci++;
    m.verts.resize(ci);
    for (int64_t v = 0; v < nv; v++)
        if (used[v] >= 0) m.verts[used[v]] = {xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]};
    for (int64_t t = 0; t < nt; t++) {
        m.tris.push_back({{used[tri[3 * t]], used[tri[3 * t + 1]], used[tri[3 * t + 2]]}});
        m.tri_tags.push_back(tags ? tags[t] : 0);
    }
    auto mk = [](int64_t a, int64_t b) { return std::make_pair(std::min(a, b), std::max(a, b)); };
    for (auto& t : m.tris) {
        m.edges.push_back(mk(t.v[0], t.v[1]));
        m.edges.push_back(mk(t.v[1], t.v[2]));
        m.edges.push_back(mk(t.v[2], t.v[0]));
    }
    std::sort(m.edges.begin(), m.edges.end());
    m.edges.erase(std::unique(m.edges.begin(), m.edges.end()), m.edges.end());
    auto offset = [&](std::pair<int64_t, int64_t> e) -> int64_t {
        auto it = std::lower_bound(m.edges.begin(), m.edges.end(), e);
        return (it != m.edges.end() && *it == e) ? int64_t(it - m.edges.begin()) : -1;
    };
    std::vector<std::pair<int64_t, int>> bedges;
    for (int64_t c = 0; c < ncurve; c++) {
        int64_t a = used[curve[2 * c]], b = used[curve[2 * c + 1]];
        int64_t o = (a < 0 || b < 0) ? -1 : offset(mk(a, b));
        if (o < 0) return -2;
        bedges.push_back({o, curve_tags[c]});
    }
    size_t ne = m.edges.size();
    std::vector<int64_t> itm(ne, -1), itp(ne, -1);
    std::vector<int> lm(ne, -1), lp(ne, -1), hasi(ne, 0), itf(ne, 0);
    for (int64_t t = 0; t < nt; t++) {
        auto& T = m.tris[t];
        std::pair<int64_t, int64_t> le[3] = {mk(T.v[0], T.v[1]), mk(T.v[1], T.v[2]), mk(T.v[2], T.v[0])};
        for (int k = 0; k < 3; k++) {
            int64_t o = offset(le[k]);
            if (itp[o] >= 0) return -1;
            if (itm[o] >= 0) {
                if (itm[o] < t) {
                    itp[o] = t;
                    lp[o] = k;
                } else {
                    itp[o] = itm[o];
                    lp[o] = lm[o];
                    itm[o] = t;
                    lm[o] = k;
                }
            } else {
                itm[o] = t;
                lm[o] = k;
            }
        }
    }
    for (auto& be : bedges)
        if (itp[be.first] >= 0) {
            hasi[be.first] = 1;
            itf[be.first] = be.second;
        }
    const int evmap[3] = {2, 0, 1};
    int64_t mi = 0;
    for (size_t e = 0; e < ne; e++) {
        if (itp[e] < 0) continue;
        Bf bf;
        auto& Tm = m.tris[itm[e]];
        auto& Tp = m.tris[itp[e]];
        bf.Aminus = m.area(itm[e]);
        bf.Aplus = m.area(itp[e]);
        bf.itminus = itm[e];
        bf.itplus = itp[e];
        bf.pminus = m.verts[Tm.v[evmap[lm[e]]]];
        bf.pplus = m.verts[Tp.v[evmap[lp[e]]]];
        vec3 d = m.verts[m.edges[e].second] - m.verts[m.edges[e].first];
        bf.length = edge_xy ? std::hypot(d.x, d.y) : norm(d);
        bf.edge_index = int64_t(e);
        bf.matrix_index = mi++;
        bf.has_itf = hasi[e];
        bf.itf = itf[e];
        m.bfs.push_back(bf);
    }
    return int64_t(m.bfs.size());
}

// RWG table as 17 doubles per function:
// Aminus Aplus itminus itplus pminus[3] pplus[3] length edge_index matrix_index
// has_itf itf edge_v0 edge_v1
void oracle_get_rwg(void* sp, double* out) {
    State* s = (State*)sp;
    for (size_t i = 0; i < s->msh.bfs.size(); i++) {
        const Bf& b = s->msh.bfs[i];
        double* o = out + 17 * i;
        o[0] = b.Aminus; o[1] = b.Aplus; o[2] = double(b.itminus); o[3] = double(b.itplus);
        o[4] = b.pminus.x; o[5] = b.pminus.y; o[6] = b.pminus.z;
        o[7] = b.pplus.x; o[8] = b.pplus.y; o[9] = b.pplus.z;
        o[10] = b.length; o[11] = double(b.edge_index); o[12] = double(b.matrix_index);
        o[13] = b.has_itf; o[14] = b.itf;
        o[15] = double(s->msh.edges[b.edge_index].first);
        o[16] = double(s->msh.edges[b.edge_index].second);
    }
}

// dunavant() points of one triangle: out[4*k] = x, y, z, w; returns count.
int oracle_dunavant(int degree, const double* p0, const double* p1, const double* p2, double* out) {
    auto q = dunavant(size_t(degree), {p0[0], p0[1], p0[2]}, {p1[0], p1[1], p1[2]}, {p2[0], p2[1], p2[2]});
    for (size_t k = 0; k < q.size(); k++) {
        out[4 * k] = q[k].p.x; out[4 * k + 1] = q[k].p.y; out[4 * k + 2] = q[k].p.z; out[4 * k + 3] = q[k].w;
    }
    return int(q.size());
}

// compute_matrix for test functions (columns) i in [c0, c1): Z column-major,
// Z[j + (i - c0)*n] for test i, source j.
void oracle_compute_matrix_cols(void* sp, double freq, int64_t c0, int64_t c1, double* Zout) {
    State* s = (State*)sp;
    const Mesh& msh = s->msh;
    cd* Z = (cd*)Zout;
    const int64_t n = int64_t(msh.bfs.size());
    double omega = 2.0 * M_PI * freq;
    double k = omega * std::sqrt(MU0 * EPS0);
    double inv_ksq = 1. / (omega * omega * MU0 * EPS0);
    const size_t deg = s->degree;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t ii = c0; ii < c1; ii++) {
        const Bf& ibf = msh.bfs[ii];
        auto iqps_minus = msh.integrate(ibf.itminus, deg);
        auto iqps_plus = msh.integrate(ibf.itplus, deg);
        for (int64_t jj = 0; jj < n; jj++) {
            const Bf& jbf = msh.bfs[jj];
            bool split_minus = (jbf.itminus == ibf.itminus) || (jbf.itminus == ibf.itplus);
            bool split_plus = (jbf.itplus == ibf.itminus) || (jbf.itplus == ibf.itplus);
            auto jqps_minus = split_minus ? msh.integrate_subtri(jbf.itminus, deg) : msh.integrate(jbf.itminus, deg);
            auto jqps_plus = split_plus ? msh.integrate_subtri(jbf.itplus, deg) : msh.integrate(jbf.itplus, deg);
            cd entry = 0.0;
            double prodl = 0.25 * ibf.length * jbf.length * M_1_PI;
            auto block = [&](const std::vector<qpoint>& I, const std::vector<qpoint>& J, bool im, bool jm,
                             double inv_AA, double sgn) {
                for (const auto& iqp : I)
                    for (const auto& jqp : J) {
                        double v = 0.25 * dot(im ? ibf.rho_minus(iqp.p) : ibf.rho_plus(iqp.p),
                                              jm ? jbf.rho_minus(jqp.p) : jbf.rho_plus(jqp.p));
                        double sv = inv_ksq;
                        double w = iqp.w * jqp.w * inv_AA;
                        double Rij = norm(iqp.p - jqp.p);
                        cd exponent{0, -k * Rij};
                        cd g = std::exp(exponent) / Rij;
                        if (sgn > 0) entry += prodl * w * (v - sv) * g;
                        else entry -= prodl * w * (v - sv) * g;
                    }
            };
            block(iqps_minus, jqps_minus, true, true, 1. / (ibf.Aminus * jbf.Aminus), +1);
            block(iqps_minus, jqps_plus, true, false, 1. / (ibf.Aminus * jbf.Aplus), -1);
            block(iqps_plus, jqps_minus, false, true, 1. / (ibf.Aplus * jbf.Aminus), -1);
            block(iqps_plus, jqps_plus, false, false, 1. / (ibf.Aplus * jbf.Aplus), +1);
            Z[jbf.matrix_index + (ibf.matrix_index - c0) * n] = entry;
        }
    }
}

// Conditioning of each entry of compute_matrix (columns [c0, c1)): the sum of the
// magnitudes of the terms the entry's double loop adds, sum |prodl w (v - sv) g|
// over the four blocks and their quadrature pairs (same loops as above). Where the
// blocks cancel, FP64 evaluations of an entry in different orders can only agree
// to a few ulps of this sum, not of the entry itself. Mout column-major, n x (c1 - c0).
void oracle_compute_matrix_magnitudes(void* sp, double freq, int64_t c0, int64_t c1, double* Mout) {
    State* s = (State*)sp;
    const Mesh& msh = s->msh;
    const int64_t n = int64_t(msh.bfs.size());
    double omega = 2.0 * M_PI * freq;
    double inv_ksq = 1. / (omega * omega * MU0 * EPS0);
    const size_t deg = s->degree;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t ii = c0; ii < c1; ii++) {
        const Bf& ibf = msh.bfs[ii];
        auto iqps_minus = msh.integrate(ibf.itminus, deg);
        auto iqps_plus = msh.integrate(ibf.itplus, deg);
        for (int64_t jj = 0; jj < n; jj++) {
            const Bf& jbf = msh.bfs[jj];
            bool split_minus = (jbf.itminus == ibf.itminus) || (jbf.itminus == ibf.itplus);
            bool split_plus = (jbf.itplus == ibf.itminus) || (jbf.itplus == ibf.itplus);
            auto jqps_minus = split_minus ? msh.integrate_subtri(jbf.itminus, deg) : msh.integrate(jbf.itminus, deg);
            auto jqps_plus = split_plus ? msh.integrate_subtri(jbf.itplus, deg) : msh.integrate(jbf.itplus, deg);
            double mag = 0.0;
            double prodl = 0.25 * ibf.length * jbf.length * M_1_PI;
            auto block = [&](const std::vector<qpoint>& I, const std::vector<qpoint>& J, bool im, bool jm,
                             double inv_AA) {
                for (const auto& iqp : I)
                    for (const auto& jqp : J) {
                        double v = 0.25 * dot(im ? ibf.rho_minus(iqp.p) : ibf.rho_plus(iqp.p),
                                              jm ? jbf.rho_minus(jqp.p) : jbf.rho_plus(jqp.p));
                        double w = iqp.w * jqp.w * inv_AA;
                        double Rij = norm(iqp.p - jqp.p);
                        mag += std::abs(prodl * w * (v - inv_ksq)) / Rij;
                    }
            };
            block(iqps_minus, jqps_minus, true, true, 1. / (ibf.Aminus * jbf.Aminus));
            block(iqps_minus, jqps_plus, true, false, 1. / (ibf.Aminus * jbf.Aplus));
            block(iqps_plus, jqps_minus, false, true, 1. / (ibf.Aplus * jbf.Aminus));
            block(iqps_plus, jqps_plus, false, false, 1. / (ibf.Aplus * jbf.Aplus));
            Mout[jbf.matrix_index + (ibf.matrix_index - c0) * n] = mag;
        }
    }
}

void oracle_compute_matrix(void* sp, double freq, double* Zout) {
    oracle_compute_matrix_cols(sp, freq, 0, int64_t(((State*)sp)->msh.bfs.size()), Zout);
}

void oracle_compute_matrix_approx(void* sp, double freq, double* Zout) {
    State* s = (State*)sp;
    const Mesh& msh = s->msh;
    cd* Z = (cd*)Zout;
    const int64_t n = int64_t(msh.bfs.size());
    double omega = 2.0 * M_PI * freq;
    double k = omega * std::sqrt(MU0 * EPS0);
    double inv_ksq = 1. / (omega * omega * MU0 * EPS0);
    double sqrt_4pi = std::sqrt(4 * M_PI);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t ii = 0; ii < n; ii++) {
        const Bf& ibf = msh.bfs[ii];
        vec3 iTmb = msh.bar(ibf.itminus), iTpb = msh.bar(ibf.itplus);
        for (int64_t jj = 0; jj < n; jj++) {
            const Bf& jbf = msh.bfs[jj];
            vec3 jTmb = msh.bar(jbf.itminus), jTpb = msh.bar(jbf.itplus);
            auto sqrt_Am = std::sqrt(msh.area(ibf.itminus));
            auto sqrt_Ap = std::sqrt(msh.area(ibf.itplus));
            cd jk{0., k};
            cd entry = 0.0;
            auto G = [&](vec3 a, vec3 b, bool self, double sA) {
                double R = norm(a - b);
                cd e{0, -k * R};
                cd g = std::exp(e) / (4.0 * M_PI * R);
                if (self) g = 0.25 * (sqrt_4pi / sA - jk) * M_1_PI;
                return g;
            };
            double rho_cmm = dot(ibf.rho_minus(iTmb), jbf.rho_minus(jTmb));
            cd Gmm = G(iTmb, jTmb, ibf.itminus == jbf.itminus, sqrt_Am);
            entry += ibf.length * jbf.length * (0.25 * rho_cmm * Gmm - inv_ksq * Gmm);
            double rho_cmp = dot(ibf.rho_minus(iTmb), jbf.rho_plus(jTpb));
            cd Gmp = G(iTmb, jTpb, ibf.itminus == jbf.itplus, sqrt_Am);
            entry -= ibf.length * jbf.length * (0.25 * rho_cmp * Gmp - inv_ksq * Gmp);
            double rho_cpm = dot(ibf.rho_plus(iTpb), jbf.rho_minus(jTmb));
            cd Gpm = G(iTpb, jTmb, ibf.itplus == jbf.itminus, sqrt_Ap);
            entry -= ibf.length * jbf.length * (0.25 * rho_cpm * Gpm - inv_ksq * Gpm);
            double rho_cpp = dot(ibf.rho_plus(iTpb), jbf.rho_plus(jTpb));
            cd Gpp = G(iTpb, jTpb, ibf.itplus == jbf.itplus, sqrt_Ap);
            entry += ibf.length * jbf.length * (0.25 * rho_cpp * Gpp - inv_ksq * Gpp);
            Z[jbf.matrix_index + ibf.matrix_index * n] = entry;
        }
    }
}

// Delta-gap orientation; signs[n] (1.0 where untouched). Returns 1 if the
// reorientation ran, 0 if not needed, -1 on a disconnected / empty feed.
int oracle_reorient(void* sp, int n_itf, const int32_t* itf_tags, int force, double* signs) {
    State* s = (State*)sp;
    const Mesh& m = s->msh;
    struct Seg { int64_t first, second, bf; };
    bool fix_needed = false;
    std::list<Seg> edges;
    for (const Bf& b : m.bfs) {
        if (!b.has_itf) continue;
        for (int k = 0; k < n_itf; k++)
            if (b.itf == itf_tags[k]) {
                if (m.tri_tags[b.itplus] <= m.tri_tags[b.itminus]) fix_needed = true;
                edges.push_back({m.edges[b.edge_index].first, m.edges[b.edge_index].second, b.matrix_index});
            }
    }
    for (size_t i = 0; i < m.bfs.size(); i++) signs[i] = 1.0;
    if (!(fix_needed || force)) return 0;
    if (edges.empty()) return -1;
    std::list<Seg> seglist;
    seglist.push_back(edges.front());
    edges.erase(edges.begin());
    while (!edges.empty()) {
        size_t before = edges.size();
        for (auto it = edges.begin(); it != edges.end();) {
            Seg f = seglist.front(), b = seglist.back();
            auto cur = it++;
            if (cur->first == f.first) {
                seglist.push_front({cur->second, cur->first, cur->bf});
                edges.erase(cur);
            } else if (cur->second == f.first) {
                seglist.push_front({cur->first, cur->second, cur->bf});
                edges.erase(cur);
            } else if (cur->first == b.second) {
                seglist.push_back({cur->first, cur->second, cur->bf});
                edges.erase(cur);
            } else if (cur->second == b.second) {
                seglist.push_back({cur->second, cur->first, cur->bf});
                edges.erase(cur);
            }
        }
        if (edges.size() == before) return -1;
    }
    auto ebar = [&](int64_t e) { return (m.verts[m.edges[e].first] + m.verts[m.edges[e].second]) / 2.0; };
    const Bf& bf0 = m.bfs[seglist.front().bf];
    vec3 dir = m.bar(bf0.itplus) - ebar(bf0.edge_index);
    double sign = +1;
    for (auto& seg : seglist) {
        const Bf& bf = m.bfs[seg.bf];
        vec3 curdir = m.bar(bf.itplus) - ebar(bf.edge_index);
        if (dot(dir, curdir) < 0) sign *= -1;
        signs[bf.matrix_index] = sign;
        dir = curdir;
    }
    return 1;
}

void oracle_rhs_delta_gap(void* sp, double freq, int n_itf, const int32_t* itf_tags, double V0re, double V0im,
                          const double* signs, double* Vout) {
    State* s = (State*)sp;
    cd* V = (cd*)Vout;
    double omega = 2.0 * M_PI * freq;
    cd voltage(V0re, V0im);
    for (const Bf& ibf : s->msh.bfs) {
        if (!ibf.has_itf) continue;
        for (int k = 0; k < n_itf; k++)
            if (ibf.itf == itf_tags[k]) {
                cd v{0.0, -ibf.length / (omega * MU0)};
                double sign = signs ? signs[ibf.matrix_index] : 1.0;
                V[ibf.matrix_index] += v * voltage * sign;
            }
    }
}

void oracle_rhs_plane_wave(void* sp, double freq, double theta_i, double phi_i, double Ethr, double Ethi,
                           double Ephr, double Ephi_, double* Vout) {
    State* s = (State*)sp;
    const Mesh& msh = s->msh;
    cd* V = (cd*)Vout;
    double omega = 2.0 * M_PI * freq;
    auto k = omega * std::sqrt(MU0 * EPS0);
    vec3 dir{std::sin(theta_i) * std::cos(phi_i), std::sin(theta_i) * std::sin(phi_i), std::cos(theta_i)};
    vec3 th{std::cos(theta_i) * std::cos(phi_i), std::cos(theta_i) * std::sin(phi_i), -std::sin(theta_i)};
    vec3 ph{-std::sin(phi_i), std::cos(phi_i), 0.0};
    cd Eth(Ethr, Ethi), Eph(Ephr, Ephi_);
    auto compute = [&](vec3 pos, cd* E) {
        cd jk{0.0, k};
        cd E0[3] = {Eth * th.x + Eph * ph.x, Eth * th.y + Eph * ph.y, Eth * th.z + Eph * ph.z};
        cd f = std::exp(jk * dot(dir, pos));
        for (int a = 0; a < 3; a++) E[a] = E0[a] * f;
    };
    for (const Bf& ibf : msh.bfs) {
        cd v{0.0, 0.0};
        auto wminus = 0.5 * ibf.length / ibf.Aminus;
        auto wplus = 0.5 * ibf.length / ibf.Aplus;
        for (auto& qp : msh.integrate(ibf.itminus, s->degree)) {
            cd E[3];
            compute(qp.p, E);
            vec3 r = ibf.rho_minus(qp.p);
            v -= wminus * qp.w * (r.x * E[0] + r.y * E[1] + r.z * E[2]);
        }
        for (auto& qp : msh.integrate(ibf.itplus, s->degree)) {
            cd E[3];
            compute(qp.p, E);
            vec3 r = ibf.rho_plus(qp.p);
            v += wplus * qp.w * (r.x * E[0] + r.y * E[1] + r.z * E[2]);
        }
        V[ibf.matrix_index] += v / cd{0, -omega * MU0};
    }
}

// run_context lumping for solution I (n complex). Results kept in the state
// and copied to the optional outputs (nt*3, nt, nt*3 complex).
void oracle_lump(void* sp, double freq, const double* Iin, double* AJ, double* AdivJ, double* J) {
    State* s = (State*)sp;
    const Mesh& m = s->msh;
    const cd* I = (const cd*)Iin;
    size_t nt = m.tris.size();
    s->freq = freq;
    s->tri_AJ.assign(3 * nt, 0.0);
    s->tri_AdivJ.assign(nt, 0.0);
    s->tri_J.assign(3 * nt, 0.0);
    for (const Bf& bf : m.bfs) {
        vec3 bm = m.bar(bf.itminus), bp = m.bar(bf.itplus);
        double Am = m.area(bf.itminus), Ap = m.area(bf.itplus);
        cd Ie = I[bf.matrix_index];
        vec3 fm = bf.eval_minus(bm), fp = bf.eval_plus(bp);
        cd Jm[3] = {fm.x * Ie, fm.y * Ie, fm.z * Ie};
        cd Jp[3] = {fp.x * Ie, fp.y * Ie, fp.z * Ie};
        for (int a = 0; a < 3; a++) {
            s->tri_AJ[3 * bf.itminus + a] += Am * Jm[a];
            s->tri_AJ[3 * bf.itplus + a] += Ap * Jp[a];
        }
        s->tri_AdivJ[bf.itminus] += Am * bf.div_minus() * Ie;
        s->tri_AdivJ[bf.itplus] += Ap * bf.div_plus() * Ie;
        for (int a = 0; a < 3; a++) {
            s->tri_J[3 * bf.itminus + a] += Jm[a];
            s->tri_J[3 * bf.itplus + a] += Jp[a];
        }
    }
    if (AJ) std::memcpy(AJ, s->tri_AJ.data(), sizeof(cd) * 3 * nt);
    if (AdivJ) std::memcpy(AdivJ, s->tri_AdivJ.data(), sizeof(cd) * nt);
    if (J) std::memcpy(J, s->tri_J.data(), sizeof(cd) * 3 * nt);
}

// eval_fields over npts points (after oracle_lump). E, H: npts*3 complex.
void oracle_eval_fields(void* sp, int64_t npts, const double* P, double* Eout, double* Hout) {
    State* s = (State*)sp;
    const Mesh& msh = s->msh;
    const double omega = 2.0 * M_PI * s->freq;
    const double k = omega * std::sqrt(MU0 * EPS0);
    const cd jomega{0.0, omega};
    const cd jk{0.0, k};
    cd* Eo = (cd*)Eout;
    cd* Ho = (cd*)Hout;
#pragma omp parallel for schedule(static)
    for (int64_t ip = 0; ip < npts; ip++) {
        vec3 pt{P[3 * ip], P[3 * ip + 1], P[3 * ip + 2]};
        cd E[3] = {0.0, 0.0, 0.0}, H[3] = {0.0, 0.0, 0.0};
        for (size_t itri = 0; itri < msh.tris.size(); itri++) {
            const vec3 bar = msh.bar(itri);
            const vec3 vR = pt - bar;
            const double R = norm(pt - bar);
            const double _4piR = 4 * M_PI * R;
            const double _4piR3 = _4piR * R * R;
            cd jkR{0, k * R};
            cd g = (std::exp(-jkR) / _4piR);
            const cd* J = &s->tri_AJ[3 * itri];
            cd divJ = s->tri_AdivJ[itri];
            double vr[3] = {vR.x, vR.y, vR.z};
            cd t = divJ * (1.0 + jkR);
            double kR2 = std::pow(k * R, 2);
            cd pre = -jomega * MU0;
            for (int a = 0; a < 3; a++) E[a] += pre * (J[a] - t * vr[a] / kR2) * g;
            cd RcJ[3] = {vr[1] * J[2] - vr[2] * J[1], vr[2] * J[0] - vr[0] * J[2], vr[0] * J[1] - vr[1] * J[0]};
            cd gradg = -((1.0 + jkR) / _4piR3) * (s->h_physical ? std::exp(-jkR) : std::exp(jkR));
            for (int a = 0; a < 3; a++) H[a] += RcJ[a] * gradg;
        }
        for (int a = 0; a < 3; a++) {
            if (Eo) Eo[3 * ip + a] = E[a];
            if (Ho) Ho[3 * ip + a] = H[a];
        }
    }
}

int64_t oracle_num_rwg(void* sp) { return int64_t(((State*)sp)->msh.bfs.size()); }
int64_t oracle_num_tri(void* sp) { return int64_t(((State*)sp)->msh.tris.size()); }

}  // extern "C"
