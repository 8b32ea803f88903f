// Right-hand sides, current lumping and field evaluation.
//
//   update_rhs(delta_gap)   src/emw_solver.cpp:352-378
//   update_rhs(plane_wave)  src/emw_solver.cpp:380-416, plane_wave src/sources.h:34-75
//   run_context lumping     src/emw_solver.h:137-164
//   eval_fields             src/emw_postpro_common.cpp:31-66 (finite-R, exact
//                           free-space kernel; H with exp(+jkR) in compat mode)
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include <algorithm>

#include "common.cuh"
#include "dfloat.cuh"

namespace frico {

// V[i] += (-j l_i / (omega mu0)) * V0 * sign_i on RWGs whose interface tag is listed.
__global__ void k_rhs_delta_gap(int64_t n, const int32_t* __restrict__ itf, const double* __restrict__ len,
                                double omega, const int32_t* __restrict__ tags, int ntags, double2 V0,
                                const double* __restrict__ signs, double2* __restrict__ V) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    int32_t t = itf[i];
    if (t == INT32_MIN) return;
    double2 acc = V[i];
    for (int k = 0; k < ntags; k++)
        if (t == tags[k]) {
            double2 v = make_double2(0.0, -len[i] / (omega * FRICO_MU0));
            double sign = signs ? signs[i] : 1.0;
            double2 vv = cmul(v, V0);
            acc = cadd(acc, make_double2(vv.x * sign, vv.y * sign));
        }
    V[i] = acc;
}

struct PlaneWave {
    double dir[3], th[3], ph[3];
    double2 Eth, Eph;
};

// E(q) = (Eth th + Eph ph) exp(j k dir.q)
__device__ __forceinline__ void pw_field(const PlaneWave& pw, double k, const double* q, double2* E) {
    double d = pw.dir[0] * q[0] + pw.dir[1] * q[1] + pw.dir[2] * q[2];
    double s, c;
    sincos(k * d, &s, &c);
    double2 ph = make_double2(c, s);
    for (int a = 0; a < 3; a++) {
        double2 e0 = cadd(cscale(pw.Eth, pw.th[a]), cscale(pw.Eph, pw.ph[a]));
        E[a] = cmul(e0, ph);
    }
}

__global__ void k_rhs_plane_wave(int64_t n, RwgDev rw, const double* __restrict__ qp, int nq, double k,
                                 double omega, PlaneWave pw, double2* __restrict__ V) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const double l = rw.len[i];
    const double wminus = 0.5 * l / rw.am[i];
    const double wplus = 0.5 * l / rw.ap[i];
    double2 v = make_double2(0.0, 0.0);
    for (int side = 0; side < 2; side++) {
        const int64_t t = side == 0 ? rw.itm[i] : rw.itp[i];
        const double* pf = side == 0 ? rw.vm + 3 * i : rw.vp + 3 * i;
        const double wside = side == 0 ? wminus : wplus;
        for (int q = 0; q < nq; q++) {
            const double* x = qp + 4 * (t * nq + q);
            double2 E[3];
            pw_field(pw, k, x, E);
            double2 dotv = make_double2(0.0, 0.0);
            for (int a = 0; a < 3; a++) dotv = cadd(dotv, cscale(E[a], x[a] - pf[a]));
            double2 term = cscale(dotv, wside * x[3]);
            v = side == 0 ? csub(v, term) : cadd(v, term);
        }
    }
    // v / (0 - j omega mu0) = (-v.im, v.re) / (omega mu0)
    const double a = omega * FRICO_MU0;
    V[i] = cadd(V[i], make_double2(-v.y / a, v.x / a));
}

// Current lumping: per triangle, contributions of its (<= 3) RWGs in
// increasing matrix index, as run_context accumulates them.
__global__ void k_lump(int64_t nt, const TriGeo* __restrict__ geo, const int32_t* __restrict__ tri_bf,
                       RwgDev rw, const double2* __restrict__ I, double2* __restrict__ AJ,
                       double2* __restrict__ AdivJ, double2* __restrict__ J) {
    int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= nt) return;
    const double* bar = geo[t].c;
    const double A = geo[t].area;
    double2 aj[3], jj[3], adj = make_double2(0, 0);
    for (int a = 0; a < 3; a++) aj[a] = jj[a] = make_double2(0, 0);
    for (int s = 0; s < 3; s++) {
        int32_t e = tri_bf[3 * t + s];
        if (e == 0) continue;
        const int64_t i = (e < 0 ? -e : e) - 1;
        const bool minus = e < 0;
        const double l = rw.len[i];
        const double area = minus ? rw.am[i] : rw.ap[i];
        const double* pf = minus ? rw.vm + 3 * i : rw.vp + 3 * i;
        const double2 Ie = I[i];
        for (int a = 0; a < 3; a++) {
            double f = minus ? (-l * (bar[a] - pf[a])) / (2.0 * area) : (l * (bar[a] - pf[a])) / (2.0 * area);
            double2 Jv = cscale(Ie, f);
            aj[a] = cadd(aj[a], cscale(Jv, A));
            jj[a] = cadd(jj[a], Jv);
        }
        double div = minus ? -l / area : l / area;
        adj = cadd(adj, cscale(Ie, A * div));
    }
    for (int a = 0; a < 3; a++) {
        AJ[3 * t + a] = aj[a];
        J[3 * t + a] = jj[a];
    }
    AdivJ[t] = adj;
}

static const int kFP = 128;   // points per CTA
static const int kFT = 128;   // triangles staged per shared-memory round

// Partial E/H sums for a block of points over one chunk of triangles.
// part[(chunk * npts + p) * 6 + {Ex,Ey,Ez,Hx,Hy,Hz}]
template <bool WITH_H>
__global__ void __launch_bounds__(kFP) k_fields_part(int64_t npts, const double* __restrict__ P, int64_t nt,
                                                    int64_t tri_per_chunk, const TriGeo* __restrict__ geo,
                                                    const double2* __restrict__ AJ,
                                                    const double2* __restrict__ AdivJ, double k, double omega,
                                                    int hphase_physical, double2* __restrict__ part) {
    __shared__ double sb[kFT][3];
    __shared__ double2 sj[kFT][4];
    const int64_t p = blockIdx.x * int64_t(kFP) + threadIdx.x;
    const int64_t t0 = blockIdx.y * tri_per_chunk;
    const int64_t t1 = min(nt, t0 + tri_per_chunk);
    double px = 0, py = 0, pz = 0;
    if (p < npts) { px = P[3 * p]; py = P[3 * p + 1]; pz = P[3 * p + 2]; }
    double2 E[3], H[3];
    for (int a = 0; a < 3; a++) E[a] = H[a] = make_double2(0, 0);
    const double2 mjwmu = make_double2(-0.0 * FRICO_MU0, -omega * FRICO_MU0);  // (-j omega) * MU0
    const double invk2 = 1.0 / (k * k);
    for (int64_t tb = t0; tb < t1; tb += kFT) {
        const int cnt = int(min(int64_t(kFT), t1 - tb));
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const double* c = geo[tb + q].c;
            sb[q][0] = c[0]; sb[q][1] = c[1]; sb[q][2] = c[2];
            sj[q][0] = AJ[3 * (tb + q)];
            sj[q][1] = AJ[3 * (tb + q) + 1];
            sj[q][2] = AJ[3 * (tb + q) + 2];
            sj[q][3] = AdivJ[tb + q];
        }
        __syncthreads();
        if (p < npts)
            for (int q = 0; q < cnt; q++) {
                const double vx = px - sb[q][0], vy = py - sb[q][1], vz = pz - sb[q][2];
                const double R = sqrt(vx * vx + vy * vy + vz * vz);
                // one division per pair: 1/(4 pi R), 1/(4 pi R^3) and 1/(kR)^2 from 1/R
                const double invR = 1.0 / R;
                const double inv4piR = invR * (0.25 * M_1_PI);
                const double inv4piR3 = inv4piR * invR * invR;
                const double kR = k * R;
                double s, c;
                sincos(kR, &s, &c);
                const double2 g = make_double2(c * inv4piR, -s * inv4piR);
                const double2 J0 = sj[q][0], J1 = sj[q][1], J2 = sj[q][2];
                const double2 t = cmul(sj[q][3], make_double2(1.0, kR));  // divJ*(1+jkR)
                const double invkR2 = invR * invR * invk2;
                const double vr[3] = {vx, vy, vz};
                const double2 Jv[3] = {J0, J1, J2};
                for (int a = 0; a < 3; a++) {
                    double2 tv = cscale(t, vr[a] * invkR2);
                    double2 d = csub(Jv[a], tv);
                    E[a] = cadd(E[a], cmul(cmul(mjwmu, d), g));
                }
                if (WITH_H) {
                    // gradg = -((1+jkR)/_4piR3) * exp(+-jkR)
                    const double2 ph = hphase_physical ? make_double2(c, -s) : make_double2(c, s);
                    const double2 gg = cmul(make_double2(-inv4piR3, -kR * inv4piR3), ph);
                    const double2 rc[3] = {csub(cscale(J2, vy), cscale(J1, vz)), csub(cscale(J0, vz), cscale(J2, vx)),
                                           csub(cscale(J1, vx), cscale(J0, vy))};
                    for (int a = 0; a < 3; a++) H[a] = cadd(H[a], cmul(rc[a], gg));
                }
            }
    }
    if (p < npts) {
        double2* o = part + (blockIdx.y * npts + p) * 6;
        for (int a = 0; a < 3; a++) { o[a] = E[a]; o[3 + a] = H[a]; }
    }
}

// The same partial sums in double-float for the mixed path (dfloat.cuh): the
// point-centroid vector and R^2 from FP64 differences, then sqrt, 1/R,
// sincos(kR) and every product and sum in double-float. With
// G = exp(-jkR) / (4 pi R), w = 1/(kR)^2 + j/(kR) (that is (1 + jkR)/(kR)^2) and
// U = divJ w G:  E_a += -j w mu (J_a G - v_a U),  H_a += (v x J)_a gg with
// gg = -(1 + jkR) exp(+-jkR) / (4 pi R^3). Currents are split once per triangle
// when staged. A pair outside the double-float range (kR >= 6400, R^2 beyond
// the split's exponents) is summed in FP64.
template <bool WITH_H>
__global__ void __launch_bounds__(kFP) k_fields_part_df(int64_t npts, const double* __restrict__ P, int64_t nt,
                                                       int64_t tri_per_chunk, const TriGeo* __restrict__ geo,
                                                       const double2* __restrict__ AJ,
                                                       const double2* __restrict__ AdivJ, double k, double omega,
                                                       int hphase_physical, double2* __restrict__ part) {
    __shared__ double sb[kFT][3];
    __shared__ float4 sj[kFT][4];      // J0, J1, J2, divJ as (re hi, re lo, im hi, im lo)
    __shared__ double2 sjd[kFT][4];    // the same in FP64 (out-of-range pairs)
    __shared__ int s_bad[kFT];
    const int64_t p = blockIdx.x * int64_t(kFP) + threadIdx.x;
    const int64_t t0 = blockIdx.y * tri_per_chunk;
    const int64_t t1 = min(nt, t0 + tri_per_chunk);
    double px = 0, py = 0, pz = 0;
    if (p < npts) { px = P[3 * p]; py = P[3 * p + 1]; pz = P[3 * p + 2]; }
    int kb = 0;
    const dfl kd = df_from_double(k, kb), invk = df_from_double(1.0 / k, kb);
    const dfl inv4pi = df_from_double(0.25 * M_1_PI, kb);
    const dfl zero = dmk(0.f);
    cdf E[3], H[3];
    for (int a = 0; a < 3; a++) E[a] = H[a] = cdf{zero, zero};
    double2 Ed[3], Hd[3];   // FP64 sums of out-of-range pairs
    for (int a = 0; a < 3; a++) Ed[a] = Hd[a] = make_double2(0, 0);
    for (int64_t tb = t0; tb < t1; tb += kFT) {
        const int cnt = int(min(int64_t(kFT), t1 - tb));
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const double* c = geo[tb + q].c;
            sb[q][0] = c[0]; sb[q][1] = c[1]; sb[q][2] = c[2];
            int bad = 0;
            for (int a = 0; a < 3; a++) {
                sjd[q][a] = AJ[3 * (tb + q) + a];
                sj[q][a] = f4_of(sjd[q][a], bad);
            }
            sjd[q][3] = AdivJ[tb + q];
            sj[q][3] = f4_of(sjd[q][3], bad);
            s_bad[q] = bad;
        }
        __syncthreads();
        if (p < npts)
            for (int q = 0; q < cnt; q++) {
                const double vx = px - sb[q][0], vy = py - sb[q][1], vz = pz - sb[q][2];
                const double r2 = fma(vx, vx, fma(vy, vy, vz * vz));
                int bad = kb | s_bad[q];
                const dfl v[3] = {df_from_double(vx, bad), df_from_double(vy, bad), df_from_double(vz, bad)};
                const dfl R = df_sqrt(df_from_double(r2, bad));
                dfl sn, cs;
                if (!bad && df_sincos(df_mul(kd, R), sn, cs)) {
                    const dfl invR = df_rcp(R);
                    const dfl i4R = df_mul(invR, inv4pi);
                    const cdf G{df_mul(cs, i4R), df_neg(df_mul(sn, i4R))};
                    const dfl ikR = df_mul(invR, invk);
                    const cdf w{df_mul(ikR, ikR), ikR};
                    const cdf U = cdf_mul(cdf_of(sj[q][3]), cdf_mul(w, G));
#pragma unroll
                    for (int a = 0; a < 3; a++)
                        E[a] = cdf_add(E[a], cdf_sub(cdf_mul(cdf_of(sj[q][a]), G), cdf_scale(U, v[a])));
                    if (WITH_H) {
                        const dfl i4R3 = df_mul(i4R, df_mul(invR, invR));
                        const dfl kR = df_mul(kd, R);
                        const cdf ph{cs, hphase_physical ? df_neg(sn) : sn};
                        // -(1 + jkR) ph / (4 pi R^3)
                        const cdf gg = cdf_scale(cdf_mul(cdf{dmk(-1.f), df_neg(kR)}, ph), i4R3);
                        const cdf J0 = cdf_of(sj[q][0]), J1 = cdf_of(sj[q][1]), J2 = cdf_of(sj[q][2]);
                        const cdf rc[3] = {cdf_sub(cdf_scale(J2, v[1]), cdf_scale(J1, v[2])),
                                           cdf_sub(cdf_scale(J0, v[2]), cdf_scale(J2, v[0])),
                                           cdf_sub(cdf_scale(J1, v[0]), cdf_scale(J0, v[1]))};
#pragma unroll
                        for (int a = 0; a < 3; a++) H[a] = cdf_add(H[a], cdf_mul(rc[a], gg));
                    }
                } else {
                    // FP64, as k_fields_part (without the -j w mu factor, applied at the end)
                    const double R64 = sqrt(r2), invR = 1.0 / R64, i4R = invR * (0.25 * M_1_PI), kR = k * R64;
                    double s, c;
                    sincos(kR, &s, &c);
                    const double2 g = make_double2(c * i4R, -s * i4R);
                    const double2 t = cmul(sjd[q][3], make_double2(1.0, kR));
                    const double ikR2 = invR * invR / (k * k);
                    const double vr[3] = {vx, vy, vz};
                    for (int a = 0; a < 3; a++) Ed[a] = cadd(Ed[a], cmul(csub(sjd[q][a], cscale(t, vr[a] * ikR2)), g));
                    if (WITH_H) {
                        const double i4R3 = i4R * invR * invR;
                        const double2 ph = hphase_physical ? make_double2(c, -s) : make_double2(c, s);
                        const double2 gg = cmul(make_double2(-i4R3, -kR * i4R3), ph);
                        const double2 J0 = sjd[q][0], J1 = sjd[q][1], J2 = sjd[q][2];
                        const double2 rc[3] = {csub(cscale(J2, vy), cscale(J1, vz)), csub(cscale(J0, vz), cscale(J2, vx)),
                                               csub(cscale(J1, vx), cscale(J0, vy))};
                        for (int a = 0; a < 3; a++) Hd[a] = cadd(Hd[a], cmul(rc[a], gg));
                    }
                }
            }
    }
    if (p < npts) {
        const double2 mjwmu = make_double2(-0.0 * FRICO_MU0, -omega * FRICO_MU0);  // (-j omega) * MU0
        double2* o = part + (blockIdx.y * npts + p) * 6;
        for (int a = 0; a < 3; a++) {
            const double2 e = cadd(make_double2(df_to_double(E[a].r), df_to_double(E[a].i)), Ed[a]);
            o[a] = cmul(mjwmu, e);
            o[3 + a] = cadd(make_double2(df_to_double(H[a].r), df_to_double(H[a].i)), Hd[a]);
        }
    }
}

__global__ void k_fields_reduce(int64_t npts, int nchunks, const double2* __restrict__ part,
                                double2* __restrict__ out) {
    int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= npts * 6) return;
    double2 acc = make_double2(0, 0);
    for (int c = 0; c < nchunks; c++) acc = cadd(acc, part[int64_t(c) * npts * 6 + idx]);
    out[idx] = acc;
}

// ------------------------------------------------------------------ host side
static RwgDev rwg_of(frico_gpu_ctx* ctx) {
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

int rhs_delta_gap(frico_gpu_ctx* ctx, double freq, int col, int n_itf, const int32_t* tags, double2 V0,
                  const double* signs) {
    int rc;
    const int64_t n = ctx->n;
    const double omega = 2.0 * M_PI * freq;
    // tags and signs go through one small device buffer
    size_t bytes = sizeof(int32_t) * std::max(1, n_itf) + 16 + (signs ? sizeof(double) * n : 0);
    DevBuf& tmp = ctx->fld_pts;
    if ((rc = ensure(ctx, tmp, bytes))) return rc;
    int32_t* dtags = (int32_t*)tmp.p;
    double* dsigns = signs ? (double*)((char*)tmp.p + ((sizeof(int32_t) * std::max(1, n_itf) + 15) & ~size_t(15))) : nullptr;
    if (n_itf > 0 && (rc = cuda_check(ctx, cudaMemcpyAsync(dtags, tags, sizeof(int32_t) * n_itf,
                                                          cudaMemcpyHostToDevice, ctx->stream), "tags")))
        return rc;
    if (signs && (rc = cuda_check(ctx, cudaMemcpyAsync(dsigns, signs, sizeof(double) * n, cudaMemcpyHostToDevice,
                                                       ctx->stream), "signs")))
        return rc;
    k_rhs_delta_gap<<<unsigned((n + 255) / 256), 256, 0, ctx->stream>>>(
        n, (const int32_t*)ctx->rwg_itf.p, (const double*)ctx->rwg_len.p, omega, dtags, n_itf, V0, dsigns,
        (double2*)ctx->rhs.p + int64_t(col) * n);
    count_launch(ctx);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "k_rhs_delta_gap"))) return rc;
    return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "rhs sync");
}

int rhs_plane_wave(frico_gpu_ctx* ctx, double freq, int col, double theta, double phi, double2 Eth, double2 Eph) {
    int rc;
    if (ctx->geo_degree != ctx->opt.degree)
        if ((rc = build_quadrature(ctx))) return rc;
    const int64_t n = ctx->n;
    const double omega = 2.0 * M_PI * freq;
    const double k = omega * std::sqrt(FRICO_MU0 * FRICO_EPS0);
    PlaneWave pw;
    pw.dir[0] = std::sin(theta) * std::cos(phi);
    pw.dir[1] = std::sin(theta) * std::sin(phi);
    pw.dir[2] = std::cos(theta);
    pw.th[0] = std::cos(theta) * std::cos(phi);
    pw.th[1] = std::cos(theta) * std::sin(phi);
    pw.th[2] = -std::sin(theta);
    pw.ph[0] = -std::sin(phi);
    pw.ph[1] = std::cos(phi);
    pw.ph[2] = 0.0;
    pw.Eth = Eth;
    pw.Eph = Eph;
    k_rhs_plane_wave<<<unsigned((n + 127) / 128), 128, 0, ctx->stream>>>(
        n, rwg_of(ctx), (const double*)ctx->qp.p, ctx->nq, k, omega, pw, (double2*)ctx->rhs.p + int64_t(col) * n);
    count_launch(ctx);
    return cuda_check(ctx, cudaGetLastError(), "k_rhs_plane_wave");
}

int lump_currents(frico_gpu_ctx* ctx, int col) {
    int rc;
    const int64_t nt = ctx->nt, n = ctx->n;
    if ((rc = ensure(ctx, ctx->tri_aj, sizeof(double2) * 3 * nt))) return rc;
    if ((rc = ensure(ctx, ctx->tri_adivj, sizeof(double2) * nt))) return rc;
    if ((rc = ensure(ctx, ctx->tri_j, sizeof(double2) * 3 * nt))) return rc;
    k_lump<<<unsigned((nt + 127) / 128), 128, 0, ctx->stream>>>(
        nt, (const TriGeo*)ctx->trigeo.p, (const int32_t*)ctx->tri_bf.p, rwg_of(ctx),
        (const double2*)ctx->sol.p + int64_t(col) * n, (double2*)ctx->tri_aj.p, (double2*)ctx->tri_adivj.p,
        (double2*)ctx->tri_j.p);
    count_launch(ctx);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "k_lump"))) return rc;
    ctx->lumped_col = col;
    return FRICO_GPU_OK;
}

// Partial-sum kernel for the context's precision: double-float for the mixed path
// (its results are checked against the FP64 path to 1e-12), FP64 for the drop-in.
static void launch_fields_part(frico_gpu_ctx* ctx, dim3 grid, cudaStream_t st, bool with_h, int64_t npts,
                               const double* P, int64_t nt, int64_t tpc, double k, double omega, double2* part) {
    const TriGeo* geo = (const TriGeo*)ctx->trigeo.p;
    const double2* aj = (const double2*)ctx->tri_aj.p;
    const double2* adj = (const double2*)ctx->tri_adivj.p;
    const int hp = ctx->opt.h_phase_mode == FRICO_HPHASE_PHYSICAL;
    const bool df = ctx->opt.precision == FRICO_PREC_MIXED;
    if (df && with_h)
        k_fields_part_df<true><<<grid, kFP, 0, st>>>(npts, P, nt, tpc, geo, aj, adj, k, omega, hp, part);
    else if (df)
        k_fields_part_df<false><<<grid, kFP, 0, st>>>(npts, P, nt, tpc, geo, aj, adj, k, omega, hp, part);
    else if (with_h)
        k_fields_part<true><<<grid, kFP, 0, st>>>(npts, P, nt, tpc, geo, aj, adj, k, omega, hp, part);
    else
        k_fields_part<false><<<grid, kFP, 0, st>>>(npts, P, nt, tpc, geo, aj, adj, k, omega, hp, part);
}

int eval_fields_dev(frico_gpu_ctx* ctx, int col, int64_t npts, const double* P_host, double2* E_host,
                    double2* H_host) {
    int rc;
    if (ctx->lumped_col != col)
        if ((rc = lump_currents(ctx, col))) return rc;
    const int64_t nt = ctx->nt;
    const double omega = 2.0 * M_PI * ctx->freq;
    const double k = omega * std::sqrt(FRICO_MU0 * FRICO_EPS0);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t pblocks = (npts + kFP - 1) / kFP;
    // Enough (point block x triangle chunk) CTAs for ~24 per SM (the pair loop is a
    // long FP64 dependency chain: occupancy hides it), chunks of >= 16 triangles.
    int64_t nchunks = std::max<int64_t>(1, (int64_t(24) * sms + pblocks - 1) / pblocks);
    nchunks = std::min<int64_t>(nchunks, std::max<int64_t>(1, nt / 16));
    const int64_t tpc = (nt + nchunks - 1) / nchunks;
    nchunks = (nt + tpc - 1) / tpc;
    if ((rc = ensure(ctx, ctx->fld_part, sizeof(double2) * 6 * npts * nchunks))) return rc;
    if ((rc = ensure(ctx, ctx->fld_out, sizeof(double2) * 6 * npts))) return rc;
    DevBuf& pts = ctx->fld_pts;
    if ((rc = ensure(ctx, pts, sizeof(double) * 3 * npts))) return rc;
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(pts.p, P_host, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice,
                                              ctx->stream), "points")))
        return rc;
    launch_fields_part(ctx, dim3(unsigned(pblocks), unsigned(nchunks)), ctx->stream, H_host != nullptr, npts,
                       (const double*)pts.p, nt, tpc, k, omega, (double2*)ctx->fld_part.p);
    k_fields_reduce<<<unsigned((npts * 6 + 255) / 256), 256, 0, ctx->stream>>>(
        npts, int(nchunks), (const double2*)ctx->fld_part.p, (double2*)ctx->fld_out.p);
    count_launch(ctx, 2);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "fields kernels"))) return rc;
    if (E_host || H_host) {
        std::vector<double2> h(6 * npts);
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(h.data(), ctx->fld_out.p, sizeof(double2) * 6 * npts,
                                                  cudaMemcpyDeviceToHost, ctx->stream), "fields out")))
            return rc;
        if ((rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "fields sync"))) return rc;
        for (int64_t p = 0; p < npts; p++)
            for (int a = 0; a < 3; a++) {
                if (E_host) E_host[3 * p + a] = h[6 * p + a];
                if (H_host) H_host[3 * p + a] = h[6 * p + 3 + a];
            }
    }
    return FRICO_GPU_OK;
}

// ------------------------------------------------------------------ allocation-free field evaluation
// Callers that cannot let the library allocate device memory in the middle of
// their work use eval_fields_noalloc: an application whose own memory pool owns
// (nearly) all of the device, or a post-processing loop that must not pay for
// cudaMalloc's device-wide synchronisation on every new size. The points and the
// fields are the caller's device buffers, and the per-chunk partial sums of
// k_fields_part go to the fixed scratch array below, compiled into the library
// (4 MiB: npts * chunks <= kNoAllocScratch / 6). Nothing in the scratch has to
// start at zero: k_fields_part writes every (chunk, point) slot that
// k_fields_reduce_split reads in the same call. The scratch is one array per
// device, shared by every context: calls whose kernels overlap on the GPU (two
// contexts, two streams) race on it.
static const int64_t kNoAllocScratch = int64_t(1) << 18;   // double2 elements
static __device__ __align__(256) double2 g_fields_scratch[kNoAllocScratch];

static std::mutex g_scratch_mu;
static const int kMaxDevices = 64;
static double2* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_fields_scratch on ctx->device (the current device).
// Looked up once per device, on the first call for that device.
static int fields_scratch(frico_gpu_ctx* ctx, double2** out) {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return set_err(ctx, FRICO_GPU_EINVAL, "eval_fields_noalloc: device ordinal out of range");
    if (!g_scratch_ptr[ctx->device]) {
        void* p = nullptr;
        int rc = cuda_check(ctx, cudaGetSymbolAddress(&p, g_fields_scratch), "cudaGetSymbolAddress(fields scratch)");
        if (rc) return rc;
        g_scratch_ptr[ctx->device] = (double2*)p;
    }
    *out = g_scratch_ptr[ctx->device];
    return FRICO_GPU_OK;
}

// E[3p + a] = sum over chunks of part[(c * npts + p) * 6 + a], H likewise (a + 3).
__global__ void k_fields_reduce_split(int64_t npts, int nchunks, const double2* __restrict__ part,
                                      double2* __restrict__ E, double2* __restrict__ H) {
    int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= npts * 6) return;
    double2 acc = make_double2(0, 0);
    for (int c = 0; c < nchunks; c++) acc = cadd(acc, part[int64_t(c) * npts * 6 + idx]);
    const int64_t p = idx / 6;
    const int a = int(idx - p * 6);
    if (a < 3) {
        if (E) E[3 * p + a] = acc;
    } else if (H) {
        H[3 * p + a - 3] = acc;
    }
}

int64_t eval_fields_noalloc_max_points() { return kNoAllocScratch / 6; }

int eval_fields_noalloc(frico_gpu_ctx* ctx, int col, int64_t npts, const double* P_dev, double2* E_dev,
                        double2* H_dev) {
    if (npts > eval_fields_noalloc_max_points())
        return set_err(ctx, FRICO_GPU_EINVAL,
                       "eval_fields_noalloc: npts = " + std::to_string(npts) + " exceeds the fixed scratch limit of " +
                           std::to_string(eval_fields_noalloc_max_points()) + " points");
    if (ctx->lumped_col != col)
        return set_err(ctx, FRICO_GPU_ESTATE,
                       "eval_fields_noalloc: currents of this column are not lumped (call frico_gpu_lump_currents)");
    int rc;
    double2* part = nullptr;
    if ((rc = fields_scratch(ctx, &part))) return rc;
    const int64_t nt = ctx->nt;
    const double omega = 2.0 * M_PI * ctx->freq;
    const double k = omega * std::sqrt(FRICO_MU0 * FRICO_EPS0);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t pblocks = (npts + kFP - 1) / kFP;
    // the same chunking as eval_fields_dev, capped by the scratch size
    int64_t nchunks = std::max<int64_t>(1, (int64_t(8) * sms + pblocks - 1) / pblocks);
    nchunks = std::min<int64_t>(nchunks, std::max<int64_t>(1, nt / 64));
    nchunks = std::min<int64_t>(nchunks, kNoAllocScratch / (6 * npts));
    const int64_t tpc = (nt + nchunks - 1) / nchunks;
    nchunks = (nt + tpc - 1) / tpc;
    launch_fields_part(ctx, dim3(unsigned(pblocks), unsigned(nchunks)), ctx->stream, H_dev != nullptr, npts, P_dev, nt,
                       tpc, k, omega, part);
    k_fields_reduce_split<<<unsigned((npts * 6 + 255) / 256), 256, 0, ctx->stream>>>(npts, int(nchunks), part, E_dev,
                                                                                     H_dev);
    count_launch(ctx, 2);
    return cuda_check(ctx, cudaGetLastError(), "fields kernels (noalloc)");
}

}  // namespace frico
