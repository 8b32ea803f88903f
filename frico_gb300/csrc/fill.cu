// EFIE impedance-matrix fill (FRICO compute_matrix / compute_matrix_approx).
//
// Reference: src/emw_solver.cpp:45-142 (quadrature fill) and :144-220 (MOM3D
// centroid fill). FRICO loops over RWG pairs (i, j) and, for each of the four
// triangle blocks (T_i-/+, T_j-/+), evaluates the Green function at every pair
// of quadrature points. The same Green value is therefore recomputed for every
// RWG pair that shares a triangle pair (9x at degree 1).
//
// GB300 layout of the same arithmetic:
//   phase 1  gtab: one Green evaluation per ordered triangle pair (a, b)
//            (degree 1: g = exp(-jkR)/R; degree >= 2: 8 weighted moments of g),
//            stored row-major [a][b] in HBM (Nt^2 * 16 B at degree 1).
//   phase 1' split moments: for every RWG i and side s the two blocks whose
//            source triangle is T_i- or T_i+ use integrate_subtri on the
//            source (src/emw_solver.cpp:67-78); their 8 moments are computed
//            once per (i, s, source) with FP64 throughout.
//   phase 2  assembly: one thread per Z entry (row j, column i); a CTA owns a
//            run of rows of one column, so stores are coalesced and the
//            column's RWG data is a broadcast. Each block is rebuilt from the
//            table with FRICO's own expression
//               entry += prodl * w * (v - 1/k^2) * g      (:81-137)
//            or, for split / higher-degree blocks, from the moments
//               F = 1/4 (Mpq - u.Mp - v.Mq + (v.u) M0) - M0/k^2
//            which is the same double sum expanded about the two centroids.
#include <cuda_runtime.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "dunavant_rules.h"

namespace frico {

__constant__ double c_orbits[160][5];
__constant__ int c_first[21];

// ------------------------------------------------------------------ geometry
__device__ __forceinline__ double dnorm3(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

// area_triangle_kahan, src/quadratures.cpp:41-57
__device__ double kahan_area(const double* p0, const double* p1, const double* p2) {
    double l10 = dnorm3(p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]);
    double l20 = dnorm3(p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]);
    double l21 = dnorm3(p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]);
    // sort ascending
    double s0 = l10, s1 = l20, s2 = l21, t;
    if (s1 < s0) { t = s0; s0 = s1; s1 = t; }
    if (s2 < s1) { t = s1; s1 = s2; s2 = t; }
    if (s1 < s0) { t = s0; s0 = s1; s1 = t; }
    double a = s2, b = s1, c = s0;
    return 0.25 * sqrt((a + (b + c)) * (c - (a - b)) * (c + (a - b)) * (a + (b - c)));
}

// dunavant(degree, p0, p1, p2), src/quadratures.cpp:321-372: writes the points
// in FRICO's permutation order; returns the number written. out[4*k] = x,y,z,w.
__device__ int dunavant_points(int degree, const double* p0, const double* p1, const double* p2,
                               double* out) {
    int rule = degree == 0 ? 0 : degree - 1;
    double area = kahan_area(p0, p1, p2);
    int k = 0;
    for (int e = c_first[rule]; e < c_first[rule + 1]; e++) {
        int perms = int(c_orbits[e][0]);
        double l0 = c_orbits[e][1], l1 = c_orbits[e][2], l2 = c_orbits[e][3], w = c_orbits[e][4] * area;
        double L[6][3];
        int np;
        if (perms == 1) {
            L[0][0] = l0; L[0][1] = l1; L[0][2] = l2; np = 1;
        } else if (perms == 3) {
            L[0][0] = l0; L[0][1] = l1; L[0][2] = l2;
            L[1][0] = l1; L[1][1] = l2; L[1][2] = l0;
            L[2][0] = l1; L[2][1] = l0; L[2][2] = l2; np = 3;
        } else {
            L[0][0] = l0; L[0][1] = l1; L[0][2] = l2;
            L[1][0] = l0; L[1][1] = l2; L[1][2] = l1;
            L[2][0] = l1; L[2][1] = l0; L[2][2] = l2;
            L[3][0] = l1; L[3][1] = l2; L[3][2] = l0;
            L[4][0] = l2; L[4][1] = l0; L[4][2] = l1;
            L[5][0] = l2; L[5][1] = l1; L[5][2] = l0; np = 6;
        }
        for (int q = 0; q < np; q++) {
            for (int d = 0; d < 3; d++)
                out[4 * k + d] = __dadd_rn(__dadd_rn(__dmul_rn(p0[d], L[q][0]), __dmul_rn(p1[d], L[q][1])),
                                           __dmul_rn(p2[d], L[q][2]));
            out[4 * k + 3] = w;
            k++;
        }
    }
    return k;
}

// Per triangle: geometry, integrate() points and integrate_subtri() points
// (src/quadratures.cpp:2678-2702): sub-triangles (v0,v1,c), (v1,v2,c), (v2,v0,c).
__global__ void k_build_quadrature(int64_t nt, const double* __restrict__ xyz,
                                   const int64_t* __restrict__ tri, int degree, int nq,
                                   TriGeo* __restrict__ geo, double* __restrict__ qp,
                                   double* __restrict__ qps) {
    int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= nt) return;
    double p[3][3];
    for (int k = 0; k < 3; k++)
        for (int d = 0; d < 3; d++) p[k][d] = xyz[3 * tri[3 * t + k] + d];
    TriGeo g;
    for (int k = 0; k < 3; k++)
        for (int d = 0; d < 3; d++) g.v[3 * k + d] = p[k][d];
    // barycenter: (p0 + p1 + p2) / 3.0, src/geom_mesh.cpp:64-69
    for (int d = 0; d < 3; d++) g.c[d] = __ddiv_rn(__dadd_rn(__dadd_rn(p[0][d], p[1][d]), p[2][d]), 3.0);
    double e0[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
    double e1[3] = {p[2][0] - p[1][0], p[2][1] - p[1][1], p[2][2] - p[1][2]};
    double cx = e0[1] * e1[2] - e0[2] * e1[1], cy = e0[2] * e1[0] - e0[0] * e1[2],
           cz = e0[0] * e1[1] - e0[1] * e1[0];
    g.area = 0.5 * dnorm3(cx, cy, cz);
    g.area_kahan = kahan_area(p[0], p[1], p[2]);
    g.pad[0] = g.pad[1] = 0.0;
    geo[t] = g;
    dunavant_points(degree, p[0], p[1], p[2], qp + 4 * nq * t);
    double* o = qps + 12 * nq * t;
    o += 4 * dunavant_points(degree, p[0], p[1], g.c, o);
    o += 4 * dunavant_points(degree, p[1], p[2], g.c, o);
    dunavant_points(degree, p[2], p[0], g.c, o);
}

// Per-RWG data used by the assembly. `a_m`/`a_p` depend on the fill mode:
//   mode 0 (degree 1): rho at the single quadrature point, q - p_free
//   mode 2 (MOM3D):    rho at the barycentre, c - p_free
// `v_m`/`v_p` = p_free - centroid, the offsets the moment expansion needs.
// The factors of a block are regrouped per half-basis (RWG i on side s), so
// that an entry costs a few FP64 FMAs per block:
//   prodl * w_p w_q / (A_is A_jt) = (q_is w_p)(q_jt w_q),  q = l / (2 sqrt(pi) A)
//   1/4 rho_is.rho_jt - 1/k^2     = rho'_is.rho'_jt - 1/k^2,  rho' = rho / 2
// (the same products as src/emw_solver.cpp:81-93, associated differently).
struct BasisAsm {
    int32_t itm, itp;
    double len;
    double a_m[3], a_p[3];   // rho'/2 at the degree-1 point (mode 0) or barycentre (mode 2), halved
    double v_m[3], v_p[3];   // p_free - centroid (moment expansion)
    double q_m, q_p;         // l / (2 sqrt(pi) A)
    double h_m, h_p;         // q * (degree-1 quadrature weight)
    // signed, pre-multiplied forms for the symmetric mode-0 assembly: with
    // u = s h a, hs = s h, hk = -s h / k^2 (s = -1 on T-, +1 on T+), a block is
    // s_a s_b h h (a.a - 1/k^2) = u_ia.u_jb + hk_ia hs_jb
    double u_m[3], u_p[3];
    double hs_m, hs_p, hk_m, hk_p;
};

// The signed factors of the mode-0 assembly as double-float pairs (hi, lo), for
// the assembly on the FP32 pipe; bad: some factor is outside the split's range,
// and the entries of this RWG take the FP64 path.
struct BasisDF {
    int32_t itm, itp;
    float um[3][2], up[3][2];
    float hsm[2], hsp[2], hkm[2], hkp[2];
    int32_t bad;
};

// dfo's triangle numbers are tnew's (the double-float table's) when tnew is given.
__global__ void k_basis_aux(int64_t n, RwgDev rw, const TriGeo* __restrict__ geo,
                            const double* __restrict__ qp, int nq, int mode, double inv_ksq,
                            BasisAsm* __restrict__ out, BasisDF* __restrict__ dfo,
                            const int32_t* __restrict__ tnew) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    BasisAsm b;
    b.itm = rw.itm[i];
    b.itp = rw.itp[i];
    b.len = rw.len[i];
    const double am = rw.am[i], ap = rw.ap[i];
    const double* qm = qp + 4 * nq * int64_t(b.itm);
    const double* qpp = qp + 4 * nq * int64_t(b.itp);
    for (int d = 0; d < 3; d++) {
        double vm = rw.vm[3 * i + d], vp = rw.vp[3 * i + d];
        if (mode == 2) {
            b.a_m[d] = 0.5 * (geo[b.itm].c[d] - vm);
            b.a_p[d] = 0.5 * (geo[b.itp].c[d] - vp);
        } else {
            b.a_m[d] = 0.5 * (qm[d] - vm);
            b.a_p[d] = 0.5 * (qpp[d] - vp);
        }
        b.v_m[d] = vm - geo[b.itm].c[d];
        b.v_p[d] = vp - geo[b.itp].c[d];
    }
    const double s = 0.5 * b.len / sqrt(M_PI);
    b.q_m = s / am;
    b.q_p = s / ap;
    b.h_m = b.q_m * qm[3];
    b.h_p = b.q_p * qpp[3];
    b.hs_m = -b.h_m;
    b.hs_p = b.h_p;
    b.hk_m = b.h_m * inv_ksq;
    b.hk_p = -b.h_p * inv_ksq;
    for (int d = 0; d < 3; d++) {
        b.u_m[d] = b.hs_m * b.a_m[d];
        b.u_p[d] = b.hs_p * b.a_p[d];
    }
    out[i] = b;
    BasisDF f;
    int bad = 0;
    f.itm = tnew ? tnew[b.itm] : b.itm;
    f.itp = tnew ? tnew[b.itp] : b.itp;
    for (int d = 0; d < 3; d++) {
        split_df(b.u_m[d], f.um[d][0], f.um[d][1], bad);
        split_df(b.u_p[d], f.up[d][0], f.up[d][1], bad);
    }
    split_df(b.hs_m, f.hsm[0], f.hsm[1], bad);
    split_df(b.hs_p, f.hsp[0], f.hsp[1], bad);
    split_df(b.hk_m, f.hkm[0], f.hkm[1], bad);
    split_df(b.hk_p, f.hkp[0], f.hkp[1], bad);
    f.bad = bad;
    dfo[i] = f;
}

// ------------------------------------------------------------------ phase 1
struct __align__(32) QPoint { double x, y, z, w; };

// g(a, b) = exp(-j k R) / R between the single degree-1 points of a and b.
__global__ void k_gtab_deg1(int64_t nt, const QPoint* __restrict__ qp, double k,
                            double2* __restrict__ G) {
    int64_t b = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    int64_t a = blockIdx.y;
    if (b >= nt) return;
    QPoint p = qp[a], q = qp[b];
    double2 g = make_double2(0.0, 0.0);
    if (a != b) {
        double dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        double R = sqrt(dx * dx + dy * dy + dz * dz);
        double s, c;
        sincos(k * R, &s, &c);
        g = make_double2(c / R, -s / R);
    }
    G[a * nt + b] = g;
}

// MOM3D centroid Green function with the analytic self term,
// src/emw_solver.cpp:181-214.
__global__ void k_gtab_approx(int64_t nt, const TriGeo* __restrict__ geo, double k,
                              double2* __restrict__ G) {
    int64_t b = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    int64_t a = blockIdx.y;
    if (b >= nt) return;
    const double* ca = geo[a].c;
    const double* cb = geo[b].c;
    double2 g;
    if (a != b) {
        double dx = ca[0] - cb[0], dy = ca[1] - cb[1], dz = ca[2] - cb[2];
        double R = sqrt(dx * dx + dy * dy + dz * dz);
        double s, c;
        sincos(k * R, &s, &c);
        double den = 4.0 * M_PI * R;
        g = make_double2(c / den, -s / den);
    } else {
        double sqrt_4pi = sqrt(4 * M_PI);
        double sa = sqrt(geo[a].area);
        // 0.25*(sqrt_4pi/sqrt_A - jk) * M_1_PI
        g = make_double2(0.25 * (sqrt_4pi / sa) * M_1_PI, 0.25 * (-k) * M_1_PI);
    }
    G[a * nt + b] = g;
}

// Symmetric tile form of the two single-point tables above: g(a,b) = g(b,a),
// so a CTA evaluates the 32x32 pairs of tile (ta, tb), ta <= tb, and stores
// the tile and its transpose (both coalesced, through shared memory).
// APPROX = 0: degree-1 points, g = exp(-jkR)/R, zero on the diagonal (never read).
// APPROX = 1: barycentres, g = exp(-jkR)/(4 pi R), MOM3D self term on the diagonal.
template <int APPROX>
__global__ void __launch_bounds__(256) k_gtab_sym(int64_t nt, const QPoint* __restrict__ qp,
                                                 const TriGeo* __restrict__ geo, double k, double2* __restrict__ G) {
    __shared__ double pa[32][3], pb[32][3];
    __shared__ double2 tile[32][33];
    // map the linear block index onto the upper-triangular tile pairs
    const int64_t T = (nt + 31) / 32;
    int64_t lin = blockIdx.x, ta = 0;
    while (lin >= T - ta) { lin -= T - ta; ta++; }
    const int64_t tb = ta + lin;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (threadIdx.x < 64) {
        int which = threadIdx.x >> 5, q = threadIdx.x & 31;
        int64_t t = (which ? tb : ta) * 32 + q;
        double* dst = which ? pb[q] : pa[q];
        if (t < nt) {
            if (APPROX) {
                dst[0] = geo[t].c[0]; dst[1] = geo[t].c[1]; dst[2] = geo[t].c[2];
            } else {
                QPoint p = qp[t];
                dst[0] = p.x; dst[1] = p.y; dst[2] = p.z;
            }
        } else {
            dst[0] = dst[1] = dst[2] = 0.0;
        }
    }
    __syncthreads();
    const double sqrt_4pi = sqrt(4 * M_PI);
    for (int r = ty; r < 32; r += 8) {
        const int64_t a = ta * 32 + r, b = tb * 32 + tx;
        double2 g = make_double2(0.0, 0.0);
        if (a < nt && b < nt) {
            if (a != b) {
                double dx = pa[r][0] - pb[tx][0], dy = pa[r][1] - pb[tx][1], dz = pa[r][2] - pb[tx][2];
                double r2 = dx * dx + dy * dy + dz * dz;
                double R = sqrt(r2);
                double s, c;
                sincos(k * R, &s, &c);
                double inv = APPROX ? 1.0 / (4.0 * M_PI * R) : 1.0 / R;
                g = make_double2(c * inv, -s * inv);
            } else if (APPROX) {
                double sa = sqrt(geo[a].area);
                g = make_double2(0.25 * (sqrt_4pi / sa) * M_1_PI, 0.25 * (-k) * M_1_PI);
            }
            G[a * nt + b] = g;
        }
        tile[r][tx] = g;
    }
    if (ta == tb) return;
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t a = tb * 32 + r, b = ta * 32 + tx;   // transposed tile
        if (a < nt && b < nt) G[a * nt + b] = tile[tx][r];
    }
}

// k_gtab_sym<0> in double-float for the mixed path: g = exp(-jkR)/R with R from
// the FP64 coordinate differences (r^2 in FP64, then split), sqrt, 1/R and
// sincos(kR) in double-float (dfloat.cuh); stored as (re hi, re lo, im hi,
// im lo). A pair outside the double-float range (kR >= 6400, r^2 beyond the
// split's exponents) is evaluated in FP64 and then split.
// Table over the renumbered triangles: entry (a, b) is the pair (told[a], told[b]).
__global__ void __launch_bounds__(256) k_gtab_sym_df(int64_t nt, const QPoint* __restrict__ qp,
                                                    const int32_t* __restrict__ told, double k,
                                                    float4* __restrict__ G) {
    __shared__ double pa[32][3], pb[32][3];
    __shared__ float4 tile[32][33];
    const int64_t T = (nt + 31) / 32;
    int64_t lin = blockIdx.x, ta = 0;
    while (lin >= T - ta) { lin -= T - ta; ta++; }
    const int64_t tb = ta + lin;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (threadIdx.x < 64) {
        int which = threadIdx.x >> 5, q = threadIdx.x & 31;
        int64_t t = (which ? tb : ta) * 32 + q;
        double* dst = which ? pb[q] : pa[q];
        if (t < nt) {
            QPoint p = qp[told[t]];
            dst[0] = p.x; dst[1] = p.y; dst[2] = p.z;
        } else {
            dst[0] = dst[1] = dst[2] = 0.0;
        }
    }
    __syncthreads();
    int kbad = 0;
    const dfl kd = df_from_double(k, kbad);
    for (int r = ty; r < 32; r += 8) {
        const int64_t a = ta * 32 + r, b = tb * 32 + tx;
        float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
        if (a < nt && b < nt) {
            if (a != b) {
                const double dx = pa[r][0] - pb[tx][0], dy = pa[r][1] - pb[tx][1], dz = pa[r][2] - pb[tx][2];
                const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
                int bad = kbad;
                const dfl R = df_sqrt(df_from_double(r2, bad));
                dfl s, c;
                if (!bad && df_sincos(df_mul(kd, R), s, c)) {
                    const dfl inv = df_rcp(R);
                    const dfl gr = df_mul(c, inv), gi = df_neg(df_mul(s, inv));
                    g = make_float4(gr.h, gr.l, gi.h, gi.l);
                } else {
                    const double Rd = sqrt(r2);
                    double sd, cd;
                    sincos(k * Rd, &sd, &cd);
                    int b2 = 0;
                    const dfl gr = df_from_double(cd / Rd, b2), gi = df_from_double(-sd / Rd, b2);
                    g = make_float4(gr.h, gr.l, gi.h, gi.l);
                }
            }
            G[a * nt + b] = g;
        }
        tile[r][tx] = g;
    }
    if (ta == tb) return;
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t a = tb * 32 + r, b = ta * 32 + tx;   // transposed tile
        if (a < nt && b < nt) G[a * nt + b] = tile[tx][r];
    }
}

// Moments of g over point sets P (test, about ca) and Q (source, about cb):
// m[0] = sum w w g, m[1..3] = sum w w g (p-ca), m[4..6] = sum w w g (q-cb),
// m[7] = sum w w g (p-ca).(q-cb).
__device__ void moments(const double* P, int np, const double* ca, const double* Q, int nq_,
                        const double* cb, double k, double2* m) {
    for (int c = 0; c < 8; c++) m[c] = make_double2(0.0, 0.0);
    for (int ip = 0; ip < np; ip++) {
        const double* p = P + 4 * ip;
        double pl[3] = {p[0] - ca[0], p[1] - ca[1], p[2] - ca[2]};
        for (int iq = 0; iq < nq_; iq++) {
            const double* q = Q + 4 * iq;
            double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
            double R = sqrt(dx * dx + dy * dy + dz * dz);
            double s, c;
            sincos(k * R, &s, &c);
            double ww = p[3] * q[3];
            double2 g = make_double2(ww * c / R, -ww * s / R);
            double ql[3] = {q[0] - cb[0], q[1] - cb[1], q[2] - cb[2]};
            double pq = pl[0] * ql[0] + pl[1] * ql[1] + pl[2] * ql[2];
            m[0] = cadd(m[0], g);
            for (int d = 0; d < 3; d++) {
                m[1 + d] = cadd(m[1 + d], cscale(g, pl[d]));
                m[4 + d] = cadd(m[4 + d], cscale(g, ql[d]));
            }
            m[7] = cadd(m[7], cscale(g, pq));
        }
    }
}

// Unsplit moments for every ordered triangle pair, degree >= 2. Planes of
// nt*nt entries: M[c*nt*nt + a*nt + b].
__global__ void k_gtab_moments(int64_t nt, const TriGeo* __restrict__ geo,
                               const double* __restrict__ qp, int nq, double k,
                               double2* __restrict__ M) {
    int64_t b = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    int64_t a = blockIdx.y;
    if (b >= nt) return;
    double2 m[8];
    if (a != b) {
        moments(qp + 4 * nq * a, nq, geo[a].c, qp + 4 * nq * b, nq, geo[b].c, k, m);
    } else {
        for (int c = 0; c < 8; c++) m[c] = make_double2(0.0, 0.0);
    }
    int64_t plane = nt * nt;
    for (int c = 0; c < 8; c++) M[c * plane + a * nt + b] = m[c];
}

// Split blocks: for RWG i, test side s (T_is, unsplit points) and source
// triangle T_it (integrate_subtri points). S[(i*4 + 2*s + t)*8 + c].
__global__ void k_split_moments(int64_t n, RwgDev rw, const TriGeo* __restrict__ geo,
                                const double* __restrict__ qp, const double* __restrict__ qps,
                                int nq, double k, double2* __restrict__ S) {
    int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= 4 * n) return;
    int64_t i = idx >> 2;
    int s = (idx >> 1) & 1, t = idx & 1;
    int64_t ta = s == 0 ? rw.itm[i] : rw.itp[i];
    int64_t tb = t == 0 ? rw.itm[i] : rw.itp[i];
    double2 m[8];
    moments(qp + 4 * nq * ta, nq, geo[ta].c, qps + 12 * nq * tb, 3 * nq, geo[tb].c, k, m);
    for (int c = 0; c < 8; c++) S[idx * 8 + c] = m[c];
}

// ------------------------------------------------------------------ phase 2
struct AsmArgs {
    int64_t n, nt, ldz;
    double inv_ksq;
    const BasisAsm* bas;
    const BasisDF* bdf;  // the same, double-float (mode 0)
    const double2* G;    // mode 0/2: [nt*nt]; mode 1: 8 planes
    const float4* G4;    // mode 0, mixed: the table in double-float (re hi, re lo, im hi, im lo), else null
    const int32_t* tnew; // with G4: G4's number of each triangle (BasisDF holds these numbers)
    const double2* S;    // split moments [n*4*8]
    double2* Z64;        // may be null
    float2* Z32;         // may be null
};

// F = 1/4 (Mpq - u.Mp - v.Mq + (v.u) M0) - M0 * inv_ksq
__device__ __forceinline__ double2 moment_block(const double2* m, int64_t stride, const double* v,
                                                const double* u, double inv_ksq) {
    double2 m0 = m[0];
    double2 acc = m[7 * stride];
    for (int d = 0; d < 3; d++) {
        acc = csub(acc, cscale(m[(1 + d) * stride], u[d]));
        acc = csub(acc, cscale(m[(4 + d) * stride], v[d]));
    }
    double vu = v[0] * u[0] + v[1] * u[1] + v[2] * u[2];
    acc = cadd(acc, cscale(m0, vu));
    return csub(cscale(acc, 0.25), cscale(m0, inv_ksq));
}

template <int MODE>
__global__ void __launch_bounds__(256) k_assemble(AsmArgs A) {
    int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    int64_t i = blockIdx.y;
    if (j >= A.n) return;
    const BasisAsm bi = A.bas[i];
    const BasisAsm bj = A.bas[j];
    double2 entry = make_double2(0.0, 0.0);
    const double lilj = bi.len * bj.len;
    const double mk = -A.inv_ksq;
#pragma unroll
    for (int blk = 0; blk < 4; blk++) {
        const int s = blk >> 1, t = blk & 1;  // order --, -+, +-, ++
        const int32_t ta = s ? bi.itp : bi.itm;
        const int32_t tb = t ? bj.itp : bj.itm;
        const double* vi = s ? bi.a_p : bi.a_m;
        const double* vj = t ? bj.a_p : bj.a_m;
        const double* oi = s ? bi.v_p : bi.v_m;
        const double* oj = t ? bj.v_p : bj.v_m;
        double2 c;
        if (MODE == 2) {
            // src/emw_solver.cpp:181-215: l_i l_j (1/4 rho.rho - 1/k^2) G
            double2 g = A.G[int64_t(ta) * A.nt + tb];
            double f = lilj * fma(vi[0], vj[0], fma(vi[1], vj[1], fma(vi[2], vj[2], mk)));
            c = cscale(g, f);
        } else {
            int split = (tb == bi.itm) ? 0 : (tb == bi.itp) ? 1 : -1;
            const double qq = (s ? bi.q_p : bi.q_m) * (t ? bj.q_p : bj.q_m);
            if (split >= 0) {
                const double2* m = A.S + (i * 4 + 2 * s + split) * 8;
                double2 F = moment_block(m, 1, oi, oj, A.inv_ksq);
                c = cscale(F, qq);
            } else if (MODE == 0) {
                // src/emw_solver.cpp:85-94: prodl w (1/4 rho.rho - 1/k^2) g
                double hh = (s ? bi.h_p : bi.h_m) * (t ? bj.h_p : bj.h_m);
                double f = hh * fma(vi[0], vj[0], fma(vi[1], vj[1], fma(vi[2], vj[2], mk)));
                double2 g = A.G[int64_t(ta) * A.nt + tb];
                c = cscale(g, f);
            } else {
                int64_t plane = A.nt * A.nt;
                double2 F = moment_block(A.G + int64_t(ta) * A.nt + tb, plane, oi, oj, A.inv_ksq);
                c = cscale(F, qq);
            }
        }
        entry = (s == t) ? cadd(entry, c) : csub(entry, c);
    }
    int64_t o = i * A.ldz + j;
    if (A.Z64) A.Z64[o] = entry;
    if (A.Z32) A.Z32[o] = make_float2(float(entry.x), float(entry.y));
}

// (Z + Z^T) / 2, src/emw_solver.h:118-120. Tiles of 32x32 above the diagonal
// and their mirror images are exchanged through shared memory.
__global__ void k_symmetrize(int64_t n, int64_t ld, double2* Z) {
    __shared__ double2 ta[32][33], tb[32][33];
    int64_t bi = blockIdx.y, bj = blockIdx.x;
    if (bj < bi) return;
    int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (int r = ty; r < 32; r += 8) {
        int64_t row = bi * 32 + r, col = bj * 32 + tx;   // tile A: rows of block bi, cols of bj
        ta[r][tx] = (row < n && col < n) ? Z[col * ld + row] : make_double2(0, 0);
        int64_t row2 = bj * 32 + r, col2 = bi * 32 + tx;  // tile B: mirror
        tb[r][tx] = (row2 < n && col2 < n) ? Z[col2 * ld + row2] : make_double2(0, 0);
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        int64_t row = bi * 32 + r, col = bj * 32 + tx;
        if (row < n && col < n) {
            double2 a = ta[r][tx], b = tb[tx][r];
            Z[col * ld + row] = make_double2((a.x + b.x) / 2.0, (a.y + b.y) / 2.0);
        }
        int64_t row2 = bj * 32 + r, col2 = bi * 32 + tx;
        if (bi != bj && row2 < n && col2 < n) {
            double2 a = tb[r][tx], b = ta[tx][r];
            Z[col2 * ld + row2] = make_double2((a.x + b.x) / 2.0, (a.y + b.y) / 2.0);
        }
    }
}

// Lower triangle <- transpose of the upper one: Z[r][c] = Z[c][r] for r > c, the
// matrix zsytrf with uplo = 'U' factors (src/lapack_wrappers.cpp:135-177).
// Block (bx, by) writes the 32 x 32 tile at rows 32 by, columns 32 bx (by >= bx)
// from the mirror tile, staged through shared memory.
__global__ void k_mirror_upper(int64_t n, int64_t ld, double2* Z) {
    __shared__ double2 t[32][33];
    const int64_t bi = blockIdx.y, bj = blockIdx.x;
    if (bi < bj) return;
    const int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 8
    for (int r = ty; r < 32; r += 8) {
        const int64_t row = bj * 32 + r, col = bi * 32 + tx;   // upper source tile
        t[r][tx] = (row < n && col < n) ? Z[col * ld + row] : make_double2(0, 0);
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t row = bi * 32 + r, col = bj * 32 + tx;
        if (row < n && col < n && row > col) Z[col * ld + row] = t[tx][r];
    }
}

// Z[j, i] of the degree-1 fill (mode 0) for basis i (column) and test j (row).
__device__ __forceinline__ double2 entry_mode0(const AsmArgs& A, const BasisAsm& bi, const BasisAsm& bj,
                                               int64_t i) {
    double2 entry = make_double2(0.0, 0.0);
#pragma unroll
    for (int blk = 0; blk < 4; blk++) {
        const int s = blk >> 1, t = blk & 1;  // order --, -+, +-, ++
        const int32_t ta = s ? bi.itp : bi.itm;
        const int32_t tb = t ? bj.itp : bj.itm;
        const int split = (tb == bi.itm) ? 0 : (tb == bi.itp) ? 1 : -1;
        if (split >= 0) {
            const double qq = (s ? bi.q_p : bi.q_m) * (t ? bj.q_p : bj.q_m);
            const double2* m = A.S + (i * 4 + 2 * s + split) * 8;
            const double2 F = moment_block(m, 1, s ? bi.v_p : bi.v_m, t ? bj.v_p : bj.v_m, A.inv_ksq);
            entry = (s == t) ? cadd(entry, cscale(F, qq)) : csub(entry, cscale(F, qq));
        } else {
            const double* ui = s ? bi.u_p : bi.u_m;
            const double* uj = t ? bj.u_p : bj.u_m;
            const double f = fma(ui[0], uj[0], fma(ui[1], uj[1], fma(ui[2], uj[2], (s ? bi.hk_p : bi.hk_m) *
                                                                                   (t ? bj.hs_p : bj.hs_m))));
            double2 g;
            if (A.G4) {
                const float4 q = A.G4[int64_t(A.tnew[ta]) * A.nt + A.tnew[tb]];
                g = make_double2(df_to_double(dmk(q.x, q.y)), df_to_double(dmk(q.z, q.w)));
            } else {
                g = A.G[int64_t(ta) * A.nt + tb];
            }
            entry.x = fma(g.x, f, entry.x);
            entry.y = fma(g.y, f, entry.y);
        }
    }
    return entry;
}

// One mode-0 entry in double-float for RWGs that share no triangle (all four
// blocks are table blocks): sum over the blocks of g_ab f_ab with
// f_ab = u_ia . u_jb + hk_ia hs_jb, the same terms as entry_mode0, from the
// double-float table; (er, ei) = the entry as (hi, lo) pairs.
__device__ __forceinline__ bool entry_mode0_df(const AsmArgs& A, const BasisDF& di, const BasisDF& dj, float2& er,
                                               float2& ei) {
    float rs = 0.f, rt = 0.f, is = 0.f, it = 0.f;
    int bad = 0;
#pragma unroll
    for (int blk = 0; blk < 4; blk++) {
        const int s = blk >> 1, t = blk & 1;
        const int32_t ta = s ? di.itp : di.itm;
        const int32_t tb = t ? dj.itp : dj.itm;
        const float(*ui)[2] = s ? di.up : di.um;
        const float(*uj)[2] = t ? dj.up : dj.um;
        const float* hk = s ? di.hkp : di.hkm;
        const float* hs = t ? dj.hsp : dj.hsm;
        float fs = 0.f, ft = 0.f;
        df_mac(fs, ft, ui[0][0], ui[0][1], uj[0][0], uj[0][1]);
        df_mac(fs, ft, ui[1][0], ui[1][1], uj[1][0], uj[1][1]);
        df_mac(fs, ft, ui[2][0], ui[2][1], uj[2][0], uj[2][1]);
        df_mac(fs, ft, hk[0], hk[1], hs[0], hs[1]);
        df_renorm(fs, ft);
        const float4 g = A.G4[int64_t(ta) * A.nt + tb];
        df_mac(rs, rt, g.x, g.y, fs, ft);
        df_mac(is, it, g.z, g.w, fs, ft);
    }
    df_renorm(rs, rt);
    df_renorm(is, it);
    er = make_float2(rs, rt);
    ei = make_float2(is, it);
    return bad == 0;
}

// Mode-0 assembly over the lower triangle of 32 x 32 tiles. Z[j, i] = Z[i, j]
// whenever RWGs i and j share no triangle (no sub-triangle split on either side:
// the Green table is symmetric and so is the block expression), so an
// off-diagonal tile is computed once and also written transposed through shared
// memory; the few pairs that share a triangle are computed in both orientations
// in FP64 (entry_mode0). The others are computed in double-float on the FP32
// pipe (entry_mode0_df; |error| about 2^-46 of sum |g f|), the FP64 value being
// the exact sum hi + lo rounded once and the complex64 one hi + lo rounded in FP32.
__global__ void __launch_bounds__(256) k_assemble_sym0(AsmArgs A) {
    const int64_t t = blockIdx.x;
    int J = int((sqrt(8.0 * double(t) + 1.0) - 1.0) * 0.5);
    while (int64_t(J) * (J + 1) / 2 > t) J--;
    while (int64_t(J + 1) * (J + 2) / 2 <= t) J++;
    const int I = int(t - int64_t(J) * (J + 1) / 2);   // I <= J
    __shared__ double2 tr[32][33];
    __shared__ float2 tr32[32][33];
    const int jl = threadIdx.x & 31, il0 = threadIdx.x >> 5;
    const int64_t j = int64_t(J) * 32 + jl;
    const bool jok = j < A.n;
    BasisDF dj;
    const BasisDF* bdf = A.bdf ? A.bdf : nullptr;
    if (jok) dj = bdf ? bdf[j] : BasisDF{A.bas[j].itm, A.bas[j].itp};
#pragma unroll 1
    for (int kk = 0; kk < 4; kk++) {
        const int il = il0 + 8 * kk;
        const int64_t i = int64_t(I) * 32 + il;
        if (jok && i < A.n) {
            const BasisDF di = bdf ? bdf[i] : BasisDF{A.bas[i].itm, A.bas[i].itp};
            const bool shared = dj.itm == di.itm || dj.itm == di.itp || dj.itp == di.itm || dj.itp == di.itp;
            double2 e;
            float2 e32;
            float2 er, ei;
            if (A.bdf && !shared && !(di.bad | dj.bad) && entry_mode0_df(A, di, dj, er, ei)) {
                e = make_double2(f2d_exact(er.x) + f2d_exact(er.y), f2d_exact(ei.x) + f2d_exact(ei.y));
                e32 = make_float2(__fadd_rn(er.x, er.y), __fadd_rn(ei.x, ei.y));
            } else {
                e = entry_mode0(A, A.bas[i], A.bas[j], i);
                e32 = make_float2(float(e.x), float(e.y));
            }
            const int64_t o = i * A.ldz + j;
            if (A.Z64) A.Z64[o] = e;
            if (A.Z32) A.Z32[o] = e32;
            if (I != J) {   // Z[i, j]
                if (shared) {
                    const double2 et = entry_mode0(A, A.bas[j], A.bas[i], j);
                    tr[il][jl] = et;
                    tr32[il][jl] = make_float2(float(et.x), float(et.y));
                } else {
                    tr[il][jl] = e;
                    tr32[il][jl] = e32;
                }
            }
        }
    }
    if (I == J) return;
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        const int r = threadIdx.x & 31, c = (threadIdx.x >> 5) + 8 * kk;
        const int64_t i = int64_t(I) * 32 + r, jj = int64_t(J) * 32 + c;
        if (i < A.n && jj < A.n) {
            const int64_t o = jj * A.ldz + i;
            if (A.Z64) A.Z64[o] = tr[r][c];
            if (A.Z32) A.Z32[o] = tr32[r][c];
        }
    }
}

__global__ void k_z64_to_z32(int64_t count, const double2* __restrict__ a, float2* __restrict__ b) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < count) b[i] = make_float2(float(a[i].x), float(a[i].y));
}

// ------------------------------------------------------------------ host side
// The Dunavant tables live in constant memory, once per device.
static int load_dunavant_tables(frico_gpu_ctx* ctx) {
    int rc = cuda_check(ctx, cudaMemcpyToSymbol(c_orbits, frico_tables::kDunavantOrbits,
                                                sizeof(frico_tables::kDunavantOrbits)),
                        "copy Dunavant table");
    if (rc) return rc;
    return cuda_check(ctx, cudaMemcpyToSymbol(c_first, frico_tables::kDunavantFirst,
                                              sizeof(frico_tables::kDunavantFirst)),
                      "copy Dunavant offsets");
}

int build_quadrature(frico_gpu_ctx* ctx) {
    int degree = ctx->opt.degree;
    if (degree < 0 || degree > frico_tables::kDunavantMaxDegree)
        return set_err(ctx, FRICO_GPU_EINVAL, "Dunavant quadrature: degree too high");
    if (int rc = device_once(ctx, kOnceDunavant, load_dunavant_tables)) return rc;
    int rule = degree == 0 ? 0 : degree - 1;
    int nq = frico_tables::kDunavantPoints[rule];
    int64_t nt = ctx->nt;
    int rc;
    if ((rc = ensure(ctx, ctx->trigeo, sizeof(TriGeo) * nt))) return rc;
    if ((rc = ensure(ctx, ctx->qp, sizeof(double) * 4 * nq * nt))) return rc;
    if ((rc = ensure(ctx, ctx->qps, sizeof(double) * 12 * nq * nt))) return rc;
    k_build_quadrature<<<unsigned((nt + 127) / 128), 128, 0, ctx->stream>>>(
        nt, (const double*)ctx->xyz.p, (const int64_t*)ctx->tri.p, degree, nq, (TriGeo*)ctx->trigeo.p,
        (double*)ctx->qp.p, (double*)ctx->qps.p);
    count_launch(ctx);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "k_build_quadrature"))) return rc;
    ctx->nq = nq;
    ctx->geo_degree = degree;
    return FRICO_GPU_OK;
}

static RwgDev rwg_dev(frico_gpu_ctx* ctx) {
    RwgDev r;
    r.itm = (int32_t*)ctx->rwg_itm.p;
    r.itp = (int32_t*)ctx->rwg_itp.p;
    r.len = (double*)ctx->rwg_len.p;
    r.am = (double*)ctx->rwg_am.p;
    r.ap = (double*)ctx->rwg_ap.p;
    r.vm = (double*)ctx->rwg_vm.p;
    r.vp = (double*)ctx->rwg_vp.p;
    r.itf = (int32_t*)ctx->rwg_itf.p;
    return r;
}

int fill_matrix(frico_gpu_ctx* ctx, double freq, bool fp64_only) {
    int rc;
    if (ctx->geo_degree != ctx->opt.degree)
        if ((rc = build_quadrature(ctx))) return rc;
    const int64_t n = ctx->n, nt = ctx->nt;
    const int nq = ctx->nq;
    const int mode = ctx->opt.approx ? 2 : (nq == 1 ? 0 : 1);
    // src/emw_solver.cpp:51-54
    const double omega = 2.0 * M_PI * freq;
    const double k = omega * std::sqrt(FRICO_MU0 * FRICO_EPS0);
    const double inv_ksq = 1. / (omega * omega * FRICO_MU0 * FRICO_EPS0);

    if ((rc = ensure(ctx, ctx->basis_aux, (sizeof(BasisAsm) + sizeof(BasisDF)) * n + 256))) return rc;
    BasisDF* bdf = (BasisDF*)(((uintptr_t)((BasisAsm*)ctx->basis_aux.p + n) + 255) & ~uintptr_t(255));
    const size_t gbytes = sizeof(double2) * size_t(nt) * size_t(nt) * (mode == 1 ? 8 : 1);
    if ((rc = ensure(ctx, ctx->gtab, gbytes))) return rc;
    if (mode != 2 && (rc = ensure(ctx, ctx->smom, sizeof(double2) * 32 * n))) return rc;
    if ((rc = ensure(ctx, ctx->z64, sizeof(double2) * size_t(n) * size_t(n)))) return rc;
    const bool want32 = ctx->opt.precision == FRICO_PREC_MIXED && !ctx->opt.force_symmetry;
    if (want32 && (rc = ensure(ctx, ctx->z32, sizeof(float2) * size_t(n) * size_t(n)))) return rc;

    RwgDev rw = rwg_dev(ctx);
    const TriGeo* geo = (const TriGeo*)ctx->trigeo.p;
    const double* qp = (const double*)ctx->qp.p;
    const double* qps = (const double*)ctx->qps.p;
    cudaStream_t st = ctx->stream;
    // double-float table and entries for the mixed path only: the FP64 drop-in (and the FP64
    // factorisation a mixed solve falls back to) keep FP64 arithmetic throughout
    const bool df = mode == 0 && ctx->opt.precision == FRICO_PREC_MIXED && !fp64_only;
    const int32_t* tnew = (const int32_t*)ctx->tri_new.p;
    k_basis_aux<<<unsigned((n + 127) / 128), 128, 0, st>>>(n, rw, geo, qp, nq, mode, inv_ksq,
                                                           (BasisAsm*)ctx->basis_aux.p, bdf, df ? tnew : nullptr);
    dim3 gt(unsigned((nt + 127) / 128), unsigned(nt));
    double2* G = (double2*)ctx->gtab.p;
    const int64_t T = (nt + 31) / 32;
    const unsigned sym_blocks = unsigned(T * (T + 1) / 2);
    if (df) {
        k_gtab_sym_df<<<sym_blocks, 256, 0, st>>>(nt, (const QPoint*)qp, (const int32_t*)ctx->tri_old.p, k,
                                                  (float4*)G);
    } else if (mode == 0) {
        k_gtab_sym<0><<<sym_blocks, 256, 0, st>>>(nt, (const QPoint*)qp, geo, k, G);
    } else if (mode == 1) {
        k_gtab_moments<<<gt, 128, 0, st>>>(nt, geo, qp, nq, k, G);
    } else {
        k_gtab_sym<1><<<sym_blocks, 256, 0, st>>>(nt, (const QPoint*)qp, geo, k, G);
    }
    if (mode != 2)
        k_split_moments<<<unsigned((4 * n + 127) / 128), 128, 0, st>>>(n, rw, geo, qp, qps, nq, k,
                                                                        (double2*)ctx->smom.p);
    AsmArgs a;
    a.n = n;
    a.nt = nt;
    a.ldz = n;
    a.inv_ksq = inv_ksq;
    a.bas = (const BasisAsm*)ctx->basis_aux.p;
    a.bdf = df ? bdf : nullptr;
    a.G4 = df ? (const float4*)G : nullptr;
    a.tnew = df ? tnew : nullptr;
    ctx->z_df = df;
    a.G = G;
    a.S = (const double2*)ctx->smom.p;
    a.Z64 = (double2*)ctx->z64.p;
    a.Z32 = want32 ? (float2*)ctx->z32.p : nullptr;
    dim3 ga(unsigned((n + 255) / 256), unsigned(n));
    const int64_t nbt = (n + 31) / 32;
    if (mode == 0) k_assemble_sym0<<<unsigned(nbt * (nbt + 1) / 2), 256, 0, st>>>(a);
    else if (mode == 1) k_assemble<1><<<ga, 256, 0, st>>>(a);
    else k_assemble<2><<<ga, 256, 0, st>>>(a);
    count_launch(ctx, mode != 2 ? 4 : 3);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "fill kernels"))) return rc;
    if (ctx->opt.force_symmetry) {
        if ((rc = symmetrize(ctx))) return rc;
        if (ctx->opt.precision == FRICO_PREC_MIXED) {
            if ((rc = ensure(ctx, ctx->z32, sizeof(float2) * size_t(n) * size_t(n)))) return rc;
            int64_t cnt = n * n;
            k_z64_to_z32<<<unsigned((cnt + 255) / 256), 256, 0, st>>>(cnt, (const double2*)ctx->z64.p,
                                                                   (float2*)ctx->z32.p);
            if ((rc = cuda_check(ctx, cudaGetLastError(), "k_z64_to_z32"))) return rc;
        }
    }
    // Algorithmic Green evaluations: ordered pairs x nq^2, plus the split blocks.
    ctx->stats.green_evals = mode == 2 ? nt * nt : nt * (nt - 1) * int64_t(nq) * nq + 4 * n * int64_t(nq) * 3 * nq;
    ctx->freq = freq;
    return FRICO_GPU_OK;
}

// Z32 <- complex64(Z64): rebuilds the mixed-precision copy (e.g. before a
// second factorisation with a different pivoting strategy).
int z64_to_z32(frico_gpu_ctx* ctx) {
    const int64_t n = ctx->n, cnt = n * n;
    int rc;
    if ((rc = ensure(ctx, ctx->z32, sizeof(float2) * size_t(cnt)))) return rc;
    k_z64_to_z32<<<unsigned((cnt + 255) / 256), 256, 0, ctx->stream>>>(cnt, (const double2*)ctx->z64.p,
                                                                       (float2*)ctx->z32.p);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_z64_to_z32");
}

int mirror_upper(frico_gpu_ctx* ctx) {
    const int64_t n = ctx->n;
    const unsigned nb = unsigned((n + 31) / 32);
    k_mirror_upper<<<dim3(nb, nb), dim3(32, 8), 0, ctx->stream>>>(n, n, (double2*)ctx->z64.p);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_mirror_upper");
}

int symmetrize(frico_gpu_ctx* ctx) {
    int64_t n = ctx->n;
    unsigned nb = unsigned((n + 31) / 32);
    k_symmetrize<<<dim3(nb, nb), dim3(32, 8), 0, ctx->stream>>>(n, n, (double2*)ctx->z64.p);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_symmetrize");
}

}  // namespace frico
