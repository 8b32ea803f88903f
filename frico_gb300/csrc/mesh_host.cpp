// Host-side mesh front end: connectivity, RWG table and delta-gap orientation.
//
// This is the one-off O(N log N) preparation FRICO does on the CPU before the
// hot loop; it stays on the host here as well. The conventions are FRICO's,
// because they fix the row/column order of Z:
//   - edges are sorted by (min vertex, max vertex) and deduplicated
//     (src/input_gmsh.cpp:129-140, edge ordering src/geom_mesh.h:35-50);
//   - for every edge, T- is the lower triangle index, T+ the higher
//     (src/input_gmsh.cpp:243-257);
//   - tagged 1-D curve segments that coincide with interior edges mark
//     interfaces (src/input_gmsh.cpp:264-269);
//   - one RWG function per interior edge in sorted-edge order, the opposite
//     vertex chosen through evmap {2,0,1} (src/rwg_basis.cpp:27-68);
//   - edge length is hypot(dx, dy) (src/geom_mesh.cpp:46-52) unless the caller
//     asks for the true 3-D length.
#include "frico_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <list>
#include <utility>
#include <vector>

namespace {

struct EdgeKey {
    int64_t a, b;  // a < b
    bool operator<(const EdgeKey& o) const { return a < o.a || (a == o.a && b < o.b); }
    bool operator==(const EdgeKey& o) const { return a == o.a && b == o.b; }
};

inline EdgeKey make_edge(int64_t u, int64_t v) { return u < v ? EdgeKey{u, v} : EdgeKey{v, u}; }

int64_t find_edge(const std::vector<EdgeKey>& edges, EdgeKey e) {
    auto it = std::lower_bound(edges.begin(), edges.end(), e);
    if (it != edges.end() && *it == e) return int64_t(it - edges.begin());
    return -1;
}

struct V3 { double x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// measure(mesh, triangle), src/geom_mesh.cpp:71-78
double tri_area(V3 p0, V3 p1, V3 p2) { return 0.5 * norm(cross(sub(p1, p0), sub(p2, p1))); }

}  // namespace

extern "C" int frico_gpu_make_function_space(int64_t nv, const double* xyz, int64_t nt,
                                             const int64_t* tri, int64_t ncurve,
                                             const int64_t* curve, const int32_t* curve_tag,
                                             int32_t edge_length_mode, frico_rwg* rwg,
                                             int64_t capacity, int64_t* n_rwg,
                                             int64_t* rwg_edge_vertices, double* vertices_out,
                                             int64_t* nv_out, int64_t* tri_out) {
    if (nv <= 0 || nt <= 0 || !xyz || !tri || !n_rwg) return FRICO_GPU_EINVAL;
    if (ncurve > 0 && (!curve || !curve_tag)) return FRICO_GPU_EINVAL;
    if (edge_length_mode != FRICO_EDGE_LENGTH_XY && edge_length_mode != FRICO_EDGE_LENGTH_TRUE)
        return FRICO_GPU_EINVAL;
    for (int64_t i = 0; i < 3 * nt; i++)
        if (tri[i] < 0 || tri[i] >= nv) return FRICO_GPU_EINVAL;
    for (int64_t i = 0; i < 2 * ncurve; i++)
        if (curve[i] < 0 || curve[i] >= nv) return FRICO_GPU_EINVAL;

    // Vertex compaction, src/input_gmsh.cpp:335-394 (monotonic renumbering,
    // so sorted-edge order is the same before and after).
    std::vector<int64_t> used(nv, -1);
    for (int64_t i = 0; i < 3 * nt; i++) used[tri[i]] = 1;
    int64_t ci = 0;
    for (int64_t v = 0; v < nv; v++)
        if (used[v] >= 0) used[v] = ci++;
    std::vector<V3> verts(ci);
    for (int64_t v = 0; v < nv; v++)
        if (used[v] >= 0) verts[used[v]] = {xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]};
    std::vector<int64_t> T(3 * nt);
    for (int64_t i = 0; i < 3 * nt; i++) T[i] = used[tri[i]];

    // Edges of every triangle: (v0,v1), (v1,v2), (v2,v0); sort + unique.
    std::vector<EdgeKey> edges;
    edges.reserve(3 * nt);
    for (int64_t t = 0; t < nt; t++) {
        const int64_t* v = &T[3 * t];
        edges.push_back(make_edge(v[0], v[1]));
        edges.push_back(make_edge(v[1], v[2]));
        edges.push_back(make_edge(v[2], v[0]));
    }
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    const int64_t ne = int64_t(edges.size());

    // Curve segments -> boundary edge pointers (lonely edge is an error).
    std::vector<std::pair<int64_t, int32_t>> bedges;
    for (int64_t s = 0; s < ncurve; s++) {
        int64_t a = curve[2 * s], b = curve[2 * s + 1];
        if (used[a] < 0 || used[b] < 0) return FRICO_GPU_EMESH;
        int64_t ofs = find_edge(edges, make_edge(used[a], used[b]));
        if (ofs < 0) return FRICO_GPU_EMESH;
        bedges.push_back({ofs, curve_tag[s]});
    }

    // compute_connectivity, src/input_gmsh.cpp:216-270.
    std::vector<int64_t> itminus(ne, -1), itplus(ne, -1);
    std::vector<int32_t> loc_m(ne, -1), loc_p(ne, -1), has_itf(ne, 0), itf(ne, 0);
    for (int64_t t = 0; t < nt; t++) {
        const int64_t* v = &T[3 * t];
        EdgeKey le[3] = {make_edge(v[0], v[1]), make_edge(v[1], v[2]), make_edge(v[2], v[0])};
        for (int k = 0; k < 3; k++) {
            int64_t ofs = find_edge(edges, le[k]);
            if (itplus[ofs] >= 0) return FRICO_GPU_EMESH;  // multiple_triangles
            if (itminus[ofs] >= 0) {
                if (itminus[ofs] < t) {
                    itplus[ofs] = t;
                    loc_p[ofs] = k;
                } else {
                    itplus[ofs] = itminus[ofs];
                    loc_p[ofs] = loc_m[ofs];
                    itminus[ofs] = t;
                    loc_m[ofs] = k;
                }
            } else {
                itminus[ofs] = t;
                loc_m[ofs] = k;
            }
        }
    }
    for (auto& be : bedges)
        if (itplus[be.first] >= 0) {
            has_itf[be.first] = 1;
            itf[be.first] = be.second;
        }

    int64_t n = 0;
    for (int64_t e = 0; e < ne; e++) n += (itplus[e] >= 0);
    *n_rwg = n;
    if (nv_out) *nv_out = ci;
    if (vertices_out)
        for (int64_t v = 0; v < ci; v++) {
            vertices_out[3 * v] = verts[v].x;
            vertices_out[3 * v + 1] = verts[v].y;
            vertices_out[3 * v + 2] = verts[v].z;
        }
    if (tri_out) std::memcpy(tri_out, T.data(), sizeof(int64_t) * 3 * nt);
    if (!rwg || capacity < n) return rwg ? FRICO_GPU_EINVAL : FRICO_GPU_OK;

    // make_function_space, src/rwg_basis.cpp:27-68.
    static const int evmap[3] = {2, 0, 1};
    int64_t mi = 0;
    for (int64_t e = 0; e < ne; e++) {
        if (itplus[e] < 0) continue;
        const int64_t* tm = &T[3 * itminus[e]];
        const int64_t* tp = &T[3 * itplus[e]];
        frico_rwg& bf = rwg[mi];
        bf.Aminus = tri_area(verts[tm[0]], verts[tm[1]], verts[tm[2]]);
        bf.Aplus = tri_area(verts[tp[0]], verts[tp[1]], verts[tp[2]]);
        bf.itminus = itminus[e];
        bf.itplus = itplus[e];
        V3 pm = verts[tm[evmap[loc_m[e]]]], pp = verts[tp[evmap[loc_p[e]]]];
        bf.pminus[0] = pm.x; bf.pminus[1] = pm.y; bf.pminus[2] = pm.z;
        bf.pplus[0] = pp.x;  bf.pplus[1] = pp.y;  bf.pplus[2] = pp.z;
        V3 d = sub(verts[edges[e].b], verts[edges[e].a]);
        bf.length = edge_length_mode == FRICO_EDGE_LENGTH_XY ? std::hypot(d.x, d.y) : norm(d);
        bf.edge_index = e;
        bf.matrix_index = mi;
        bf.has_interface = has_itf[e];
        bf.interface_tag = itf[e];
        if (rwg_edge_vertices) {
            rwg_edge_vertices[2 * mi] = edges[e].a;
            rwg_edge_vertices[2 * mi + 1] = edges[e].b;
        }
        mi++;
    }
    return FRICO_GPU_OK;
}

// reorient_deltagap_edges, src/emw_solver.cpp:222-350: chain the feed edges and
// flip signs so that adjacent RWG functions along the gap point the same way.
extern "C" int frico_gpu_reorient_deltagap(int64_t nv, const double* xyz, const int64_t* tri,
                                           const int32_t* tri_tag, int64_t n,
                                           const frico_rwg* rwg, const int64_t* rwg_edge_vertices,
                                           int32_t n_itf, const int32_t* itf_tags, int32_t force,
                                           double* signs, int32_t* applied) {
    if (nv <= 0 || !xyz || !tri || !tri_tag || n <= 0 || !rwg || !rwg_edge_vertices || !signs ||
        !applied || n_itf < 0 || (n_itf > 0 && !itf_tags))
        return FRICO_GPU_EINVAL;
    auto vtx = [&](int64_t v) { return V3{xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]}; };
    auto tri_bar = [&](int64_t t) {
        V3 a = vtx(tri[3 * t]), b = vtx(tri[3 * t + 1]), c = vtx(tri[3 * t + 2]);
        return V3{(a.x + b.x + c.x) / 3.0, (a.y + b.y + c.y) / 3.0, (a.z + b.z + c.z) / 3.0};
    };
    auto edge_bar = [&](int64_t i) {
        V3 a = vtx(rwg_edge_vertices[2 * i]), b = vtx(rwg_edge_vertices[2 * i + 1]);
        return V3{(a.x + b.x) / 2.0, (a.y + b.y) / 2.0, (a.z + b.z) / 2.0};
    };
    *applied = 0;
    for (int64_t i = 0; i < n; i++) signs[i] = 1.0;

    struct Seg { int64_t first, second, bf; };
    std::list<Seg> edges;  // (iv0, iv1, matrix index)
    bool fix_needed = false;
    for (int64_t i = 0; i < n; i++) {
        if (!rwg[i].has_interface) continue;
        for (int32_t k = 0; k < n_itf; k++)
            if (rwg[i].interface_tag == itf_tags[k]) {
                if (tri_tag[rwg[i].itplus] <= tri_tag[rwg[i].itminus]) fix_needed = true;
                edges.push_back({rwg_edge_vertices[2 * i], rwg_edge_vertices[2 * i + 1],
                                 rwg[i].matrix_index});
            }
    }
    if (!(fix_needed || force)) return FRICO_GPU_OK;
    if (edges.empty()) return FRICO_GPU_EINVAL;

    std::list<Seg> chain;
    chain.push_back(edges.front());
    edges.pop_front();
    while (!edges.empty()) {
        size_t before = edges.size();
        for (auto it = edges.begin(); it != edges.end();) {
            Seg f = chain.front(), b = chain.back();
            auto cur = it++;
            // At most one of the four cases applies to a well-formed chain.
            if (cur->first == f.first) {
                chain.push_front({cur->second, cur->first, cur->bf});
                edges.erase(cur);
            } else if (cur->second == f.first) {
                chain.push_front({cur->first, cur->second, cur->bf});
                edges.erase(cur);
            } else if (cur->first == b.second) {
                chain.push_back({cur->first, cur->second, cur->bf});
                edges.erase(cur);
            } else if (cur->second == b.second) {
                chain.push_back({cur->second, cur->first, cur->bf});
                edges.erase(cur);
            }
        }
        if (edges.size() == before) return FRICO_GPU_EINVAL;  // not connected
    }

    const Seg& s0 = chain.front();
    V3 dir = sub(tri_bar(rwg[s0.bf].itplus), edge_bar(s0.bf));
    double sign = 1.0;
    for (auto& s : chain) {
        V3 curdir = sub(tri_bar(rwg[s.bf].itplus), edge_bar(s.bf));
        if (dot(dir, curdir) < 0) sign *= -1.0;
        signs[rwg[s.bf].matrix_index] = sign;
        dir = curdir;
    }
    *applied = 1;
    return FRICO_GPU_OK;
}
