// Fields of many right-hand sides at once: eval_fields (src/emw_postpro_common.cpp:31-90)
// over a set of RHS columns, for the multi-incidence workloads (monostatic /
// many-angle bistatic RCS: 64 incidences x 65 341 observation points).
//
// The single-column kernel spends most of a (point, triangle) pair on the
// geometry and the Green function (sqrt, sincos, divisions); with RT columns
// per thread those are computed once and each column costs a few complex
// FMAs:  E_a += c1 AJ_a + c2_a D,  c1 = -j w mu0 g,  c2_a = -c1 (1 + jkR) vR_a / (kR)^2,
//        H_a += (vR x AJ)_a gg,  gg = -(1 + jkR) e^{+-jkR} / (4 pi R^3).
// (the same products as the single-column kernel, associated per pair).
// Threads: one observation point x RT columns; grid.z walks column tiles,
// grid.y splits the triangles when the other two dimensions leave SMs idle.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "common.cuh"
#include "dfloat.cuh"

namespace frico {

namespace {

constexpr int kMP = 128;   // points per CTA
constexpr int kMT = 64;    // triangles staged per step
constexpr int kRT = 4;     // RHS columns per thread

template <bool WITH_H>
__global__ void __launch_bounds__(kMP) k_fields_multi(int64_t npts, const double* __restrict__ P, int64_t nt,
                                                      int64_t tri_per_chunk, const TriGeo* __restrict__ geo,
                                                      const double2* __restrict__ AJ, const double2* __restrict__ AD,
                                                      int ncols, double k, double omega, int hphase_physical,
                                                      double2* __restrict__ part) {
    __shared__ double sc[kMT][3];
    __shared__ double2 sj[kMT][kRT][4];
    const int64_t p = blockIdx.x * int64_t(kMP) + threadIdx.x;
    const int c0 = blockIdx.z * kRT;
    const int64_t t0 = blockIdx.y * tri_per_chunk, t1 = min(nt, t0 + tri_per_chunk);
    double px = 0, py = 0, pz = 0;
    if (p < npts) { px = P[3 * p]; py = P[3 * p + 1]; pz = P[3 * p + 2]; }
    double2 E[kRT][3], H[kRT][3];
#pragma unroll
    for (int r = 0; r < kRT; r++)
#pragma unroll
        for (int a = 0; a < 3; a++) E[r][a] = H[r][a] = make_double2(0, 0);
    const double2 mjwmu = make_double2(-0.0 * FRICO_MU0, -omega * FRICO_MU0);
    const double invk2 = 1.0 / (k * k);
    for (int64_t tb = t0; tb < t1; tb += kMT) {
        const int cnt = int(min(int64_t(kMT), t1 - tb));
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += kMP) {
            const double* c = geo[tb + q].c;
            sc[q][0] = c[0];
            sc[q][1] = c[1];
            sc[q][2] = c[2];
#pragma unroll
            for (int r = 0; r < kRT; r++) {
                const int col = c0 + r;
                if (col < ncols) {
                    const double2* aj = AJ + (int64_t(col) * nt + tb + q) * 3;
                    sj[q][r][0] = aj[0];
                    sj[q][r][1] = aj[1];
                    sj[q][r][2] = aj[2];
                    sj[q][r][3] = AD[int64_t(col) * nt + tb + q];
                } else {
                    sj[q][r][0] = sj[q][r][1] = sj[q][r][2] = sj[q][r][3] = make_double2(0, 0);
                }
            }
        }
        __syncthreads();
        if (p < npts)
            for (int q = 0; q < cnt; q++) {
                const double vx = px - sc[q][0], vy = py - sc[q][1], vz = pz - sc[q][2];
                const double R = sqrt(vx * vx + vy * vy + vz * vz);
                // one division per pair: 1/(4 pi R), 1/(4 pi R^3) and 1/(kR)^2 from 1/R
                const double invR = 1.0 / R;
                const double inv4piR = invR * (0.25 * M_1_PI);
                const double kR = k * R;
                double s, c;
                sincos(kR, &s, &c);
                const double2 g = make_double2(c * inv4piR, -s * inv4piR);
                const double2 c1 = cmul(mjwmu, g);
                // -c1 (1 + jkR) / kR^2
                const double2 m = cscale(cmul(c1, make_double2(1.0, kR)), -(invR * invR * invk2));
                const double vr[3] = {vx, vy, vz};
                double2 c2[3];
#pragma unroll
                for (int a = 0; a < 3; a++) c2[a] = cscale(m, vr[a]);
                double2 gv[3];
                if (WITH_H) {
                    const double inv4piR3 = inv4piR * invR * invR;
                    const double2 ph = hphase_physical ? make_double2(c, -s) : make_double2(c, s);
                    const double2 gg = cmul(make_double2(-inv4piR3, -kR * inv4piR3), ph);
#pragma unroll
                    for (int a = 0; a < 3; a++) gv[a] = cscale(gg, vr[a]);
                }
#pragma unroll
                for (int r = 0; r < kRT; r++) {
                    const double2 J0 = sj[q][r][0], J1 = sj[q][r][1], J2 = sj[q][r][2], D = sj[q][r][3];
                    const double2 Jv[3] = {J0, J1, J2};
#pragma unroll
                    for (int a = 0; a < 3; a++) E[r][a] = cadd(E[r][a], cadd(cmul(c1, Jv[a]), cmul(c2[a], D)));
                    if (WITH_H) {
                        // (vR x J) gg = gv x J
                        H[r][0] = cadd(H[r][0], csub(cmul(gv[1], J2), cmul(gv[2], J1)));
                        H[r][1] = cadd(H[r][1], csub(cmul(gv[2], J0), cmul(gv[0], J2)));
                        H[r][2] = cadd(H[r][2], csub(cmul(gv[0], J1), cmul(gv[1], J0)));
                    }
                }
            }
    }
    if (p < npts) {
        const int nper = WITH_H ? 6 : 3;
#pragma unroll
        for (int r = 0; r < kRT; r++) {
            const int col = c0 + r;
            if (col >= ncols) break;
            double2* o = part + ((int64_t(blockIdx.y) * ncols + col) * npts + p) * nper;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                o[a] = E[r][a];
                if (WITH_H) o[3 + a] = H[r][a];
            }
        }
    }
}

// The same in double-float for the mixed path (dfloat.cuh): R^2 from FP64
// differences, then sqrt, 1/R, sincos(kR) and every product and sum in
// double-float; currents split once per staged triangle. A pair outside the
// double-float range (kR >= 6400, R^2 beyond the split's exponents) is summed in FP64.
template <bool WITH_H>
__global__ void __launch_bounds__(kMP) k_fields_multi_df(int64_t npts, const double* __restrict__ P, int64_t nt,
                                                         int64_t tri_per_chunk, const TriGeo* __restrict__ geo,
                                                         const double2* __restrict__ AJ, const double2* __restrict__ AD,
                                                         int ncols, double k, double omega, int hphase_physical,
                                                         double2* __restrict__ part) {
    __shared__ double sc[kMT][3];
    __shared__ float4 sj[kMT][kRT][4];
    __shared__ int s_bad[kMT];
    const int64_t p = blockIdx.x * int64_t(kMP) + threadIdx.x;
    const int c0 = blockIdx.z * kRT;
    const int64_t t0 = blockIdx.y * tri_per_chunk, t1 = min(nt, t0 + tri_per_chunk);
    double px = 0, py = 0, pz = 0;
    if (p < npts) { px = P[3 * p]; py = P[3 * p + 1]; pz = P[3 * p + 2]; }
    int kb = 0;
    const dfl kd = df_from_double(k, kb), invk = df_from_double(1.0 / k, kb);
    const dfl wmu = df_from_double(omega * FRICO_MU0, kb), inv4pi = df_from_double(0.25 * M_1_PI, kb);
    const dfl zero = dmk(0.f);
    cdf E[kRT][3], H[kRT][3];
#pragma unroll
    for (int r = 0; r < kRT; r++)
#pragma unroll
        for (int a = 0; a < 3; a++) E[r][a] = H[r][a] = cdf{zero, zero};
    const double2 mjwmu = make_double2(-0.0 * FRICO_MU0, -omega * FRICO_MU0);
    const double invk2 = 1.0 / (k * k);
    for (int64_t tb = t0; tb < t1; tb += kMT) {
        const int cnt = int(min(int64_t(kMT), t1 - tb));
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += kMP) {
            const double* c = geo[tb + q].c;
            sc[q][0] = c[0];
            sc[q][1] = c[1];
            sc[q][2] = c[2];
            int bad = 0;
#pragma unroll
            for (int r = 0; r < kRT; r++) {
                const int col = c0 + r;
                if (col < ncols) {
                    const double2* aj = AJ + (int64_t(col) * nt + tb + q) * 3;
                    sj[q][r][0] = f4_of(aj[0], bad);
                    sj[q][r][1] = f4_of(aj[1], bad);
                    sj[q][r][2] = f4_of(aj[2], bad);
                    sj[q][r][3] = f4_of(AD[int64_t(col) * nt + tb + q], bad);
                } else {
                    sj[q][r][0] = sj[q][r][1] = sj[q][r][2] = sj[q][r][3] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
            s_bad[q] = bad;
        }
        __syncthreads();
        if (p < npts)
            for (int q = 0; q < cnt; q++) {
                const double vx = px - sc[q][0], vy = py - sc[q][1], vz = pz - sc[q][2];
                const double r2 = fma(vx, vx, fma(vy, vy, vz * vz));
                int bad = kb;
                const dfl v[3] = {df_from_double(vx, bad), df_from_double(vy, bad), df_from_double(vz, bad)};
                const dfl R = df_sqrt(df_from_double(r2, bad));
                dfl sn, cs;
                if (!bad && !s_bad[q] && df_sincos(df_mul(kd, R), sn, cs)) {
                    const dfl invR = df_rcp(R), i4R = df_mul(invR, inv4pi);
                    const cdf g{df_mul(cs, i4R), df_neg(df_mul(sn, i4R))};
                    const cdf c1{df_mul(wmu, g.i), df_neg(df_mul(wmu, g.r))};   // -j w mu g
                    const dfl ikR = df_mul(invR, invk), kR = df_mul(kd, R);
                    // m = -c1 (1 + jkR) / (kR)^2
                    const cdf m = cdf_scale(cdf_mul(c1, cdf{dmk(-1.f), df_neg(kR)}), df_mul(ikR, ikR));
                    const cdf c2[3] = {cdf_scale(m, v[0]), cdf_scale(m, v[1]), cdf_scale(m, v[2])};
                    cdf gv[3];
                    if (WITH_H) {
                        const dfl i4R3 = df_mul(i4R, df_mul(invR, invR));
                        const cdf ph{cs, hphase_physical ? df_neg(sn) : sn};
                        const cdf gg = cdf_scale(cdf_mul(cdf{dmk(-1.f), df_neg(kR)}, ph), i4R3);
#pragma unroll
                        for (int a = 0; a < 3; a++) gv[a] = cdf_scale(gg, v[a]);
                    }
#pragma unroll
                    for (int r = 0; r < kRT; r++) {
                        const cdf J0 = cdf_of(sj[q][r][0]), J1 = cdf_of(sj[q][r][1]), J2 = cdf_of(sj[q][r][2]);
                        const cdf D = cdf_of(sj[q][r][3]);
                        const cdf Jv[3] = {J0, J1, J2};
#pragma unroll
                        for (int a = 0; a < 3; a++) E[r][a] = cdf_add(E[r][a], cdf_add(cdf_mul(c1, Jv[a]), cdf_mul(c2[a], D)));
                        if (WITH_H) {
                            H[r][0] = cdf_add(H[r][0], cdf_sub(cdf_mul(gv[1], J2), cdf_mul(gv[2], J1)));
                            H[r][1] = cdf_add(H[r][1], cdf_sub(cdf_mul(gv[2], J0), cdf_mul(gv[0], J2)));
                            H[r][2] = cdf_add(H[r][2], cdf_sub(cdf_mul(gv[0], J1), cdf_mul(gv[1], J0)));
                        }
                    }
                } else {
                    // FP64 (as k_fields_multi), added into the double-float sums
                    const double R64 = sqrt(r2), invR = 1.0 / R64, i4R = invR * (0.25 * M_1_PI), kR = k * R64;
                    double s, c;
                    sincos(kR, &s, &c);
                    const double2 g = make_double2(c * i4R, -s * i4R);
                    const double2 c1 = cmul(mjwmu, g);
                    const double2 m = cscale(cmul(c1, make_double2(1.0, kR)), -(invR * invR * invk2));
                    const double vr[3] = {vx, vy, vz};
                    double2 gv[3];
                    if (WITH_H) {
                        const double i4R3 = i4R * invR * invR;
                        const double2 ph = hphase_physical ? make_double2(c, -s) : make_double2(c, s);
                        const double2 gg = cmul(make_double2(-i4R3, -kR * i4R3), ph);
                        for (int a = 0; a < 3; a++) gv[a] = cscale(gg, vr[a]);
                    }
#pragma unroll
                    for (int r = 0; r < kRT; r++) {
                        const int col = c0 + r;
                        if (col >= ncols) continue;
                        const double2* aj = AJ + (int64_t(col) * nt + tb + q) * 3;
                        const double2 Jv[3] = {aj[0], aj[1], aj[2]};
                        const double2 D = AD[int64_t(col) * nt + tb + q];
                        int b2 = 0;
                        for (int a = 0; a < 3; a++) {
                            const double2 e = cadd(cmul(c1, Jv[a]), cmul(cscale(m, vr[a]), D));
                            E[r][a] = cdf_add(E[r][a], cdf_of(f4_of(e, b2)));
                        }
                        if (WITH_H) {
                            const double2 h[3] = {csub(cmul(gv[1], Jv[2]), cmul(gv[2], Jv[1])),
                                                  csub(cmul(gv[2], Jv[0]), cmul(gv[0], Jv[2])),
                                                  csub(cmul(gv[0], Jv[1]), cmul(gv[1], Jv[0]))};
                            for (int a = 0; a < 3; a++) H[r][a] = cdf_add(H[r][a], cdf_of(f4_of(h[a], b2)));
                        }
                    }
                }
            }
    }
    if (p < npts) {
        const int nper = WITH_H ? 6 : 3;
#pragma unroll
        for (int r = 0; r < kRT; r++) {
            const int col = c0 + r;
            if (col >= ncols) continue;
            double2* o = part + ((int64_t(blockIdx.y) * ncols + col) * npts + p) * nper;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                o[a] = make_double2(df_to_double(E[r][a].r), df_to_double(E[r][a].i));
                if (WITH_H) o[3 + a] = make_double2(df_to_double(H[r][a].r), df_to_double(H[r][a].i));
            }
        }
    }
}

// out[(col * npts + p) * nper + x] = sum over chunks (fixed order)
__global__ void k_fields_multi_reduce(int64_t cnt, int nchunks, const double2* __restrict__ part,
                                      double2* __restrict__ out) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= cnt) return;
    double2 acc = part[i];
    for (int c = 1; c < nchunks; c++) acc = cadd(acc, part[int64_t(c) * cnt + i]);
    out[i] = acc;
}

}  // namespace

int lump_currents(frico_gpu_ctx* ctx, int col);   // fields.cu

// E (and H) for columns [col0, col0 + ncols) at npts points (host in / host out
// buffers [ncols][npts][3]).
int eval_fields_multi(frico_gpu_ctx* ctx, int col0, int ncols, int64_t npts, const double* P_host,
                      double2* E_host, double2* H_host) {
    int rc;
    const int64_t nt = ctx->nt;
    cudaStream_t st = ctx->stream;
    if ((rc = ensure(ctx, ctx->mlump, sizeof(double2) * 4 * nt * size_t(ncols)))) return rc;
    double2* AJ = (double2*)ctx->mlump.p;
    double2* AD = AJ + 3 * nt * size_t(ncols);
    // lump each column with the single-column kernel, then gather
    for (int c = 0; c < ncols; c++) {
        if ((rc = lump_currents(ctx, col0 + c))) return rc;
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(AJ + 3 * nt * size_t(c), ctx->tri_aj.p, sizeof(double2) * 3 * nt,
                                                  cudaMemcpyDeviceToDevice, st), "gather AJ")))
            return rc;
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(AD + nt * size_t(c), ctx->tri_adivj.p, sizeof(double2) * nt,
                                                  cudaMemcpyDeviceToDevice, st), "gather AdivJ")))
            return rc;
    }
    const bool with_h = H_host != nullptr;
    const int fe = ctx->opt.fields_engine;
    // AUTO: the GEMM form on the mixed path for many columns over many (point, triangle) pairs;
    // a few points or columns (the sweep's 8 probe points) stay on the direct kernels
    const bool gemm = !with_h && (fe == FRICO_FIELDS_GEMM ||
                                  (fe == FRICO_FIELDS_AUTO && ctx->opt.precision == FRICO_PREC_MIXED && ncols >= 8 &&
                                   npts * nt >= (int64_t(1) << 24) && fields_gemm_available(ctx)));
    if (fe == FRICO_FIELDS_GEMM && !fields_gemm_available(ctx))
        return set_err(ctx, FRICO_GPU_EINVAL, "fields GEMM: tensor cores (tcgen05) not available on this device");
    if (gemm) {
        // E as tensor-core GEMMs: points and E on the device, in the field workspace
        const int64_t cnt = int64_t(ncols) * npts * 3;
        if ((rc = ensure(ctx, ctx->mfld, sizeof(double2) * cnt + sizeof(double) * 3 * npts + 256))) return rc;
        double2* Ed = (double2*)ctx->mfld.p;
        double* dP = (double*)(Ed + cnt);
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(dP, P_host, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, st),
                             "points")))
            return rc;
        if ((rc = eval_fields_gemm(ctx, ncols, npts, dP, AJ, AD, Ed, 0))) return rc;
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(E_host, Ed, sizeof(double2) * cnt, cudaMemcpyDeviceToHost, st),
                             "fields out")))
            return rc;
        return cuda_check(ctx, cudaStreamSynchronize(st), "fields sync");
    }
    const int nper = with_h ? 6 : 3;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t pblocks = (npts + kMP - 1) / kMP;
    const int64_t ctiles = (ncols + kRT - 1) / kRT;
    int64_t nchunks = std::max<int64_t>(1, (int64_t(8) * sms + pblocks * ctiles - 1) / (pblocks * ctiles));
    nchunks = std::min<int64_t>(nchunks, std::max<int64_t>(1, nt / 64));
    const int64_t tpc = (nt + nchunks - 1) / nchunks;
    nchunks = (nt + tpc - 1) / tpc;
    const int64_t cnt = int64_t(ncols) * npts * nper;
    if ((rc = ensure(ctx, ctx->mfld, sizeof(double2) * (cnt * (nchunks + 1)) + sizeof(double) * 3 * npts + 256)))
        return rc;
    double2* part = (double2*)ctx->mfld.p;
    double2* out = part + cnt * nchunks;
    double* dP = (double*)(out + cnt);
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(dP, P_host, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, st),
                         "points")))
        return rc;
    const double omega = 2.0 * M_PI * ctx->freq;
    const double k = omega * std::sqrt(FRICO_MU0 * FRICO_EPS0);
    const dim3 grid = dim3(unsigned(pblocks), unsigned(nchunks), unsigned(ctiles));
    const int hp = ctx->opt.h_phase_mode == FRICO_HPHASE_PHYSICAL;
    const TriGeo* geo = (const TriGeo*)ctx->trigeo.p;
    const bool df = ctx->opt.precision == FRICO_PREC_MIXED;   // double-float on the mixed path
    if (df && with_h)
        k_fields_multi_df<true><<<grid, kMP, 0, st>>>(npts, dP, nt, tpc, geo, AJ, AD, ncols, k, omega, hp, part);
    else if (df)
        k_fields_multi_df<false><<<grid, kMP, 0, st>>>(npts, dP, nt, tpc, geo, AJ, AD, ncols, k, omega, hp, part);
    else if (with_h)
        k_fields_multi<true><<<grid, kMP, 0, st>>>(npts, dP, nt, tpc, geo, AJ, AD, ncols, k, omega, hp, part);
    else
        k_fields_multi<false><<<grid, kMP, 0, st>>>(npts, dP, nt, tpc, geo, AJ, AD, ncols, k, omega, hp, part);
    k_fields_multi_reduce<<<unsigned((cnt + 255) / 256), 256, 0, st>>>(cnt, int(nchunks), part, out);
    count_launch(ctx, 2);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "fields_multi kernels"))) return rc;
    std::vector<double2> h(cnt);
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(h.data(), out, sizeof(double2) * cnt, cudaMemcpyDeviceToHost, st),
                         "fields out")))
        return rc;
    if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "fields sync"))) return rc;
    for (int64_t i = 0; i < int64_t(ncols) * npts; i++)
        for (int a = 0; a < 3; a++) {
            if (E_host) E_host[3 * i + a] = h[nper * i + a];
            if (H_host) H_host[3 * i + a] = h[nper * i + 3 + a];
        }
    return FRICO_GPU_OK;
}

}  // namespace frico
