// Far field of many right-hand sides as complex GEMMs on the tensor cores: the
// multi-column form of eval_fields (src/emw_postpro_common.cpp:31-90) for the
// many-incidence scattering workloads (64 incidences x 65 341 observation points).
//
// FRICO sums, per observation point P and triangle t (vR = P - c_t, R = |vR|),
//   E += -j w mu0 (AJ_t - AdivJ_t (1 + jkR) vR / (kR)^2) e^{-jkR} / (4 pi R).
// With e^{-jkR} = e^{-jk|P|} e^{-jk(R - |P|)} the point's own phase factors out
// of the sum, and with vR = P - c_t the sum splits into two matrix products over
// the triangles (K = Nt), for every current column at once:
//   G'(P, t) = e^{-jk(R - |P|)} / R,        H'(P, t) = (1 + jkR) / (kR)^2 G'(P, t)
//   S1 = G' [AJ_x AJ_y AJ_z]  (per column),  S2 = H' [AdivJ, c_x AdivJ, c_y AdivJ, c_z AdivJ]
//   E_a = -j w mu0 / (4 pi) e^{-jk|P|} (S1_a - P_a S2_0 + S2_{1+a}).
// G' and H' are generated per triangle chunk for all points (phase R - |P| and its
// sine / cosine in double-float, so the phase of a 190-radian path is exact to
// ~1e-12; the values rounded to FP32), written split into TF32 hi / lo; the
// products run on the tcgen05 3xTF32 tensor cores (gemm_tc.cu, k_gemm_dfacc) with
// the currents as the B operand; the TMEM result of every second k-step is moved
// into double-float sums (the FP32 tensor-core accumulation spans 6 MMAs only), and
// the triangle chunks add into double-float sums. The point phase e^{-jk|P|} and the final
// combination are FP64.
//
// Real-GEMM layout of the complex products (A^ real, B* doubled):
//   A^  (points x 2 Kc):  row p = (Re G'(p, t), Im G'(p, t)) over the chunk's t
//   B*  (2 ncols' x 2 Kc): row 2j = (Re B_tj, -Im B_tj), row 2j + 1 = (Im B_tj, Re B_tj)
//   (A^ B*^T)[p, 2j + s] = Re / Im of (G' B)[p, j],
// so C is real, points x 2 ncols', column-major: Re and Im of column j in the
// real columns 2j and 2j + 1.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "common.cuh"
#include "dfloat.cuh"
#include "frico_gpu_debug.h"

namespace frico {

namespace {

constexpr int kGenThreads = 128;   // triangles of a chunk per generator CTA pass
constexpr int kGenPoints = 8;      // points per generator CTA

// x rounded to the nearest TF32 value (10 explicit mantissa bits; ties away from zero),
// by integer operations on the magnitude bits
__device__ __forceinline__ float tf32_rn(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// x as hi + lo, both TF32 values, rounded to nearest: |x - hi - lo| <= 2^-22 |x| with no
// bias in sign. (Truncated splits leave lo with the sign of x, and the tensor cores'
// truncation of lo to TF32 then shrinks every product by about 5e-7 at once, a
// systematic error of the far-field sums.)
__device__ __forceinline__ void put_pair(float* hp, float* lp, int64_t o, float a, float b) {
    const float ah = tf32_rn(a), bh = tf32_rn(b);
    *reinterpret_cast<float2*>(hp + o) = make_float2(ah, bh);
    *reinterpret_cast<float2*>(lp + o) = make_float2(tf32_rn(a - ah), tf32_rn(b - bh));
}

// B* operands of every chunk: chunk c holds rows 2j, 2j + 1 for the 3 ncols columns of
// [AJ_x AJ_y AJ_z] (j = 3 col + a), then for the 4 ncols columns of
// [AdivJ, c_x AdivJ, c_y AdivJ, c_z AdivJ] (j = 3 ncols + 4 col + q); KP = 2 kc values per row.
__global__ void k_ff_bsplit(int64_t nt, int ncols, int nchunks, int kc, const TriGeo* __restrict__ geo,
                            const double2* __restrict__ AJ, const double2* __restrict__ AD, float* Bh, float* Bl) {
    const int cols = 7 * ncols, KP = 2 * kc;
    const int64_t total = int64_t(nchunks) * cols * kc;
    for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < total;
         idx += int64_t(gridDim.x) * blockDim.x) {
        const int tl = int(idx % kc);
        const int64_t rc = idx / kc;
        const int j = int(rc % cols);
        const int64_t c = rc / cols;
        const int64_t t = c * kc + tl;
        double2 v = make_double2(0.0, 0.0);
        if (t < nt) {
            if (j < 3 * ncols) {
                v = AJ[(int64_t(j / 3) * nt + t) * 3 + j % 3];
            } else {
                const int jj = j - 3 * ncols, q = jj & 3;
                const double2 d = AD[int64_t(jj >> 2) * nt + t];
                const double s = q == 0 ? 1.0 : geo[t].c[q - 1];
                v = make_double2(d.x * s, d.y * s);
            }
        }
        const float re = float(v.x), im = float(v.y);
        const int64_t row0 = (c * cols + j) * 2;
        put_pair(Bh, Bl, row0 * KP + 2 * tl, re, -im);
        put_pair(Bh, Bl, (row0 + 1) * KP + 2 * tl, im, re);
    }
}

// A^ operands of triangles [t0, t0 + kc) for points [0, np) of P (3 doubles each):
// row p of the G' and H' arrays, values 2 tl, 2 tl + 1. Thread = triangle of the
// chunk, kGenPoints points per CTA. A pair whose double-float phase is out of
// range (never for finite points a few wavelengths or more from the mesh) is
// computed in FP64 instead.
__global__ void __launch_bounds__(kGenThreads) k_ff_gen(int np, const double* __restrict__ P, int64_t nt, int64_t t0,
                                                        int kc, const TriGeo* __restrict__ geo, double k, float* Ggh,
                                                        float* Ggl, float* Ghh, float* Ghl) {
    __shared__ double sp[kGenPoints][4];
    const int KP = 2 * kc;
    const int p0 = blockIdx.x * kGenPoints;
    if (threadIdx.x < kGenPoints) {
        const int p = p0 + threadIdx.x;
        double x = 0, y = 0, z = 0;
        if (p < np) { x = P[3 * p]; y = P[3 * p + 1]; z = P[3 * p + 2]; }
        sp[threadIdx.x][0] = x;
        sp[threadIdx.x][1] = y;
        sp[threadIdx.x][2] = z;
        sp[threadIdx.x][3] = sqrt(x * x + y * y + z * z);
    }
    __syncthreads();
    int bad = 0;
    const dfl kd = df_from_double(k, bad);
    const float kf = float(k);
    for (int tl = threadIdx.x; tl < kc; tl += kGenThreads) {
        const int64_t t = t0 + tl;
        const bool live = t < nt;
        double c[3] = {0.0, 0.0, 0.0};
        if (live) { c[0] = geo[t].c[0]; c[1] = geo[t].c[1]; c[2] = geo[t].c[2]; }
        int cb = bad;
        const dfl cx = df_from_double(c[0], cb), cy = df_from_double(c[1], cb), cz = df_from_double(c[2], cb);
        for (int i = 0; i < kGenPoints; i++) {
            const int p = p0 + i;
            if (p >= np) break;
            float gr = 0.f, gi = 0.f, hr = 0.f, hi = 0.f;
            if (live) {
                int b = cb;
                const dfl dx = df_add(df_from_double(sp[i][0], b), df_neg(cx));
                const dfl dy = df_add(df_from_double(sp[i][1], b), df_neg(cy));
                const dfl dz = df_add(df_from_double(sp[i][2], b), df_neg(cz));
                const dfl R = df_sqrt(df_add(df_add(df_mul(dx, dx), df_mul(dy, dy)), df_mul(dz, dz)));
                const dfl ph = df_mul(kd, df_add(R, df_neg(df_from_double(sp[i][3], b))));   // k (R - |P|)
                const bool neg = ph.h < 0.f;
                dfl sn, cs;
                float s, co, Rf;
                if (!b && R.h > 0.f && df_sincos(neg ? df_neg(ph) : ph, sn, cs)) {
                    s = neg ? -sn.h : sn.h;
                    co = cs.h;
                    Rf = R.h;
                } else {   // FP64
                    const double vx = sp[i][0] - c[0], vy = sp[i][1] - c[1], vz = sp[i][2] - c[2];
                    const double R64 = sqrt(vx * vx + vy * vy + vz * vz);
                    double s64, c64;
                    sincos(k * (R64 - sp[i][3]), &s64, &c64);
                    s = float(s64);
                    co = float(c64);
                    Rf = float(R64);
                }
                const float invR = 1.f / Rf, ikR = 1.f / (kf * Rf);
                gr = co * invR;
                gi = -s * invR;
                // (1 + jkR) / (kR)^2 = 1 / (kR)^2 + j / (kR)
                const float a = ikR * ikR, bb = ikR;
                hr = gr * a - gi * bb;
                hi = gr * bb + gi * a;
            }
            const int64_t o = int64_t(p) * KP + 2 * tl;
            put_pair(Ggh, Ggl, o, gr, gi);
            put_pair(Ghh, Ghl, o, hr, hi);
        }
    }
}

// E[col][p0 + p][a] = -j w mu0 / (4 pi) e^{-jk|P|} (S1_a - P_a S2_0 + S2_{1+a}) for the batch.
__global__ void k_ff_finish(int np, int ncols, const double* __restrict__ P, double k, double omega,
                            const float2* __restrict__ S1, const float2* __restrict__ S2, int64_t npts_total,
                            int64_t p0, double2* __restrict__ E) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= int64_t(np) * ncols) return;
    const int p = int(i % np), col = int(i / np);
    const double px[3] = {P[3 * p], P[3 * p + 1], P[3 * p + 2]};
    const double pn = sqrt(px[0] * px[0] + px[1] * px[1] + px[2] * px[2]);
    double s, c;
    sincos(k * pn, &s, &c);
    // -j w mu0 / (4 pi) e^{-jk|P|}
    const double m = omega * FRICO_MU0 * 0.25 * M_1_PI;
    const double2 pre = make_double2(-m * s, -m * c);
    auto at = [&](const float2* S, int j) {   // complex column j, point p, from its double-float parts
        const float2 re = S[int64_t(2 * j) * np + p], im = S[int64_t(2 * j + 1) * np + p];
        return make_double2(double(re.x) + double(re.y), double(im.x) + double(im.y));
    };
    const double2 s20 = at(S2, 4 * col);
    for (int a = 0; a < 3; a++) {
        const double2 s1 = at(S1, 3 * col + a), s2 = at(S2, 4 * col + 1 + a);
        const double2 v = make_double2(s1.x - px[a] * s20.x + s2.x, s1.y - px[a] * s20.y + s2.y);
        E[(int64_t(col) * npts_total + p0 + p) * 3 + a] = cmul(pre, v);
    }
}

}  // namespace

// Triangles per launch (K = 2 kc real values per product): the chunk's G' and H' operands
// for all points of a batch are materialised, the products add into the double-float sums.
static const int kFieldsGemmKc = 512;
// k-steps (8 real values of K) per TMEM accumulator before its sum moves to double-float
static const int kFieldsGemmGroup = 2;
// diagnostic overrides of the two (frico_gpu_debug_fields_gemm_config; 0 = the defaults)
static int g_kc_override = 0, g_group_override = 0;

}  // namespace frico

extern "C" int frico_gpu_debug_fields_gemm_config(int32_t kc, int32_t group) {
    if (kc < 0 || kc % 16 != 0 || (group != 0 && group != 1 && group != 2 && group != 4)) return FRICO_GPU_EINVAL;
    frico::g_kc_override = kc;
    frico::g_group_override = group;
    return FRICO_GPU_OK;
}

namespace frico {

bool fields_gemm_available(frico_gpu_ctx* ctx) { return gemm_tc_available(ctx); }

// E for ncols columns at npts device points dP[3 * npts] into the device array
// E_dev[ncols][npts][3], from the lumped currents AJ[ncols][nt][3], AD[ncols][nt]
// (device, FP64). kc <= 0: the default chunk of triangles.
int eval_fields_gemm(frico_gpu_ctx* ctx, int ncols, int64_t npts, const double* dP, const double2* AJ,
                     const double2* AD, double2* E_dev, int kc) {
    if (kc <= 0) kc = g_kc_override > 0 ? g_kc_override : kFieldsGemmKc;
    const int group = g_group_override > 0 ? g_group_override : kFieldsGemmGroup;
    if (kc % 16 != 0) return set_err(ctx, FRICO_GPU_EINVAL, "fields GEMM: chunk must be a multiple of 16 triangles");
    cudaStream_t st = ctx->stream;
    const int64_t nt = ctx->nt;
    const int KP = 2 * kc;
    const int nchunks = int((nt + kc - 1) / kc);
    const int cols = 7 * ncols;
    // points per batch: the chunk operands (G' and H', hi and lo) and the FP64 sums of a
    // batch stay below about 2 GB
    const int64_t per_point = int64_t(4) * KP * 4 + int64_t(2) * cols * 8;
    const int64_t np_max = std::max<int64_t>(128, (int64_t(1) << 31) / per_point);
    const int64_t npb = std::min<int64_t>(npts, np_max);
    const size_t a_elems = size_t(npb) * KP;
    const size_t b_elems = size_t(nchunks) * cols * 2 * KP;
    const size_t s_elems = size_t(npb) * 2 * cols;
    auto al = [](size_t bytes) { return (bytes + 1023) & ~size_t(1023); };
    const size_t bytes = 4 * al(sizeof(float) * a_elems) + 2 * al(sizeof(float) * b_elems) +
                         al(sizeof(float2) * s_elems) + 1024;
    int rc;
    if ((rc = ensure(ctx, ctx->ffws, bytes))) return rc;
    if ((rc = ensure(ctx, ctx->status, sizeof(DeviceStatus)))) return rc;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st), "status"))) return rc;
    char* base = (char*)(((uintptr_t)ctx->ffws.p + 1023) & ~uintptr_t(1023));
    auto take = [&](size_t b) { char* p = base; base += al(b); return p; };
    float* Ggh = (float*)take(sizeof(float) * a_elems);
    float* Ggl = (float*)take(sizeof(float) * a_elems);
    float* Ghh = (float*)take(sizeof(float) * a_elems);
    float* Ghl = (float*)take(sizeof(float) * a_elems);
    float* Bh = (float*)take(sizeof(float) * b_elems);
    float* Bl = (float*)take(sizeof(float) * b_elems);
    float2* S = (float2*)take(sizeof(float2) * s_elems);   // double-float (hi, lo) sums
    const TriGeo* geo = (const TriGeo*)ctx->trigeo.p;
    {
        const int64_t total = int64_t(nchunks) * cols * kc;
        const unsigned blocks = unsigned(std::min<int64_t>((total + 255) / 256, 65535));
        k_ff_bsplit<<<blocks, 256, 0, st>>>(nt, ncols, nchunks, kc, geo, AJ, AD, Bh, Bl);
        count_launch(ctx);
    }
    const double omega = 2.0 * M_PI * ctx->freq;
    const double k = omega * std::sqrt(FRICO_MU0 * FRICO_EPS0);
    for (int64_t p0 = 0; p0 < npts; p0 += npb) {
        const int np = int(std::min<int64_t>(npb, npts - p0));
        const double* Pb = dP + 3 * p0;
        float2* S1 = S;                                  // np x 6 ncols (real), column-major
        float2* S2 = S + size_t(np) * 6 * ncols;         // np x 8 ncols
        for (int c = 0; c < nchunks; c++) {
            k_ff_gen<<<unsigned((np + kGenPoints - 1) / kGenPoints), kGenThreads, 0, st>>>(
                np, Pb, nt, int64_t(c) * kc, kc, geo, k, Ggh, Ggl, Ghh, Ghl);
            count_launch(ctx);
            const float* B1h = Bh + size_t(c) * cols * 2 * KP;
            const float* B1l = Bl + size_t(c) * cols * 2 * KP;
            const size_t b2 = size_t(6) * ncols * KP;
            if ((rc = gemm_tc_dfacc_pair(ctx, st, np, KP, group, c > 0 ? 1 : 0, S1, np, 6 * ncols, Ggh,
                                         Ggl, B1h, B1l, S2, np, 8 * ncols, Ghh, Ghl, B1h + b2, B1l + b2)))
                return rc;
        }
        const int64_t cnt = int64_t(np) * ncols;
        k_ff_finish<<<unsigned((cnt + 127) / 128), 128, 0, st>>>(np, ncols, Pb, k, omega, S1, S2, npts, p0, E_dev);
        count_launch(ctx);
        if ((rc = cuda_check(ctx, cudaGetLastError(), "fields GEMM kernels"))) return rc;
    }
    DeviceStatus hs;
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(&hs, ctx->status.p, sizeof hs, cudaMemcpyDeviceToHost, st), "status")))
        return rc;
    if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "fields GEMM sync"))) return rc;
    if (hs.err == FRICO_DEV_ERR_TIMEOUT) return set_err(ctx, FRICO_GPU_ETIMEOUT, "tensor-core GEMM wait timed out");
    return FRICO_GPU_OK;
}

}  // namespace frico
