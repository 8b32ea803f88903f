// GMRES refinement for the mixed-precision solve (GMRES-IR): when classical
// refinement with the complex64 factors contracts too slowly (kappa(Z) * eps32
// close to 1: electrically small structures, the EFIE low-frequency regime),
// the same factors become a right preconditioner for restarted flexible GMRES
// on the FP64 system Z d = r, with FP64 matrix-vector products against the resident
// Z64 and FP64 Arnoldi vectors. Each iteration costs one preconditioner apply
// (the two chained triangular solves), one FP64 product with Z and a
// classical Gram-Schmidt pass repeated once (CGS2); all right-hand sides run
// in lockstep, each with its own Hessenberg matrix and Givens rotations on the
// host. A column whose estimated residual meets the target stops taking new
// basis vectors (they are zeroed). Every restart ends with the true FP64
// residual b - Z x.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "common.cuh"

namespace frico {

int matvec_fp64(frico_gpu_ctx* ctx, const double2* X, int nrhs, double2* Y);                          // lu.cu
int matvec_z64(frico_gpu_ctx* ctx, const double2* X, int nrhs, double2* Y, bool df);                 // lu.cu
int precond_apply_fp32(frico_gpu_ctx* ctx, const double2* In, int64_t ld_in, int nrhs, double2* Out);  // lu.cu

namespace {

// dst[:, c] = scale[c] * src[:, c]
__global__ void k_scale_cols(int n, int nrhs, const double2* __restrict__ src, int64_t ld_src,
                             const double* __restrict__ scale, double2* __restrict__ dst, int64_t ld_dst) {
    const int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= int64_t(n) * nrhs) return;
    const int r = int(idx % n), c = int(idx / n);
    dst[c * ld_dst + r] = cscale(src[c * ld_src + r], scale[c]);
}

// h[c * hs + i] = sum_r conj(V_ci[r]) W_c[r]; block (i, c), V_ci = V + c ldc + i n.
__global__ void __launch_bounds__(256) k_gs_dots(int n, const double2* __restrict__ V, int64_t ldc,
                                                const double2* __restrict__ W, double2* __restrict__ h, int hs) {
    __shared__ double2 red[8];
    const int i = blockIdx.x, c = blockIdx.y;
    const double2* v = V + c * ldc + int64_t(i) * n;
    const double2* w = W + int64_t(c) * n;
    double2 acc = make_double2(0, 0);
    for (int r = threadIdx.x; r < n; r += 256) {
        const double2 a = v[r], b = w[r];
        cmac_conj(acc, a, b);
    }
    for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = red[0];
        for (int k = 1; k < 8; k++) t = cadd(t, red[k]);
        h[c * hs + i] = t;
    }
}

// W_c -= sum_{i < k} h[c hs + i] V_ci
__global__ void k_gs_axpy(int n, int nrhs, int k, const double2* __restrict__ V, int64_t ldc,
                          const double2* __restrict__ h, int hs, double2* __restrict__ W) {
    const int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= int64_t(n) * nrhs) return;
    const int r = int(idx % n), c = int(idx / n);
    double2 w = W[idx];
    for (int i = 0; i < k; i++) w = cfms(w, h[c * hs + i], V[c * ldc + int64_t(i) * n + r]);
    W[idx] = w;
}

// out[c] = ||W_c||^2
__global__ void __launch_bounds__(256) k_norm2_cols(int n, const double2* __restrict__ W, double* __restrict__ out) {
    __shared__ double red[8];
    const double2* w = W + int64_t(blockIdx.x) * n;
    double acc = 0.0;
    for (int r = threadIdx.x; r < n; r += 256) acc += w[r].x * w[r].x + w[r].y * w[r].y;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < 8; k++) t += red[k];
        out[blockIdx.x] = t;
    }
}

// D_c = sum_{i < k} y[c m + i] V_ci
__global__ void k_combine(int n, int nrhs, int k, const double2* __restrict__ V, int64_t ldc,
                          const double2* __restrict__ y, int m, double2* __restrict__ D) {
    const int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= int64_t(n) * nrhs) return;
    const int r = int(idx % n), c = int(idx / n);
    double2 acc = make_double2(0, 0);
    for (int i = 0; i < k; i++) acc = cadd(acc, cmul(y[c * m + i], V[c * ldc + int64_t(i) * n + r]));
    D[idx] = acc;
}

__global__ void k_add_to(int64_t cnt, const double2* __restrict__ U, double2* __restrict__ X) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < cnt) X[i] = cadd(X[i], U[i]);
}

__global__ void k_sub(int64_t cnt, const double2* __restrict__ B, const double2* __restrict__ Y,
                      double2* __restrict__ R) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < cnt) R[i] = csub(B[i], Y[i]);
}

using cd = std::complex<double>;

}  // namespace

int gmres_refine(frico_gpu_ctx* ctx, double2* X, const double2* B, double2* R, const double* bnorm, double tol,
                 int max_iters, int* iters_out, double* rel_out) {
    const int n = int(ctx->n), nrhs = ctx->nrhs;
    const int64_t cnt = int64_t(n) * nrhs;
    // restart length: near kappa * eps32 = 1 one Krylov space needs 40-90 vectors, and
    // how many swings by tens with the last bits of the factors; a restart loses them
    const int m = std::max(1, std::min(120, max_iters));
    const int64_t ldc = int64_t(m + 1) * n;   // column c's basis: V + c ldc, vector i at + i n
    const int64_t ldz = int64_t(m) * n;       // preconditioned basis: Zb + c ldz, vector i at + i n
    cudaStream_t st = ctx->stream;
    int rc;
    // Arnoldi products in double-float (the restarts' true residuals stay FP64)
    bool use_df = ctx->opt.residual_mode == FRICO_RESIDUAL_AUTO;
    if (use_df && (rc = cuda_check(ctx, cudaMemsetAsync(&((DeviceStatus*)ctx->status.p)->df_range, 0, sizeof(int),
                                                        st), "df flag")))
        return rc;
    const size_t vbytes = sizeof(double2) * size_t(nrhs) * (ldc + ldz);
    const size_t wbytes = sizeof(double2) * size_t(cnt);
    const size_t hbytes = sizeof(double2) * size_t(nrhs) * (m + 1);
    if ((rc = ensure(ctx, ctx->gm_ws, vbytes + 3 * wbytes + 3 * hbytes + sizeof(double) * 2 * nrhs + 1024)))
        return rc;
    double2* V = (double2*)ctx->gm_ws.p;
    double2* Zb = V + size_t(nrhs) * ldc;
    double2* U = Zb + size_t(nrhs) * ldz;
    double2* W = U + cnt;
    double2* D = W + cnt;
    double2* dh = D + cnt;                        // two CGS passes + y
    double2* dy = dh + 2 * size_t(nrhs) * (m + 1);
    double* dsc = (double*)(dy + size_t(nrhs) * (m + 1));
    double* dnr = dsc + nrhs;
    const unsigned g1 = unsigned((cnt + 255) / 256);
    std::vector<double> hnorm(nrhs), hscale(nrhs);
    std::vector<double2> hh(2 * size_t(nrhs) * (m + 1)), hy(size_t(nrhs) * (m + 1));
    auto colnorms = [&](const double2* A) -> int {
        k_norm2_cols<<<nrhs, 256, 0, st>>>(n, A, dnr);
        count_launch(ctx);
        int r2 = cuda_check(ctx, cudaMemcpyAsync(hnorm.data(), dnr, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st),
                            "gmres norms");
        if (!r2) r2 = cuda_check(ctx, cudaStreamSynchronize(st), "gmres sync");
        return r2;
    };
    int total = 0;
    double rel = 1e300;
    if ((rc = colnorms(R))) return rc;
    for (;;) {
        // restart: v_0 = r / ||r|| for the columns still above the tolerance
        std::vector<double> beta(nrhs);
        std::vector<bool> active(nrhs), done(nrhs);
        rel = 0.0;
        for (int c = 0; c < nrhs; c++) {
            beta[c] = std::sqrt(hnorm[c]);
            const double rc_rel = beta[c] / bnorm[c];
            rel = std::max(rel, rc_rel);
            active[c] = std::isfinite(rc_rel) && rc_rel > tol && beta[c] > 0;
            done[c] = !active[c];
            hscale[c] = active[c] ? 1.0 / beta[c] : 0.0;
        }
        bool any = false;
        for (int c = 0; c < nrhs; c++) any = any || active[c];
        if (!any || total >= max_iters || !std::isfinite(rel)) break;
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(dsc, hscale.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, st),
                             "gmres scale")))
            return rc;
        k_scale_cols<<<g1, 256, 0, st>>>(n, nrhs, R, n, dsc, V, ldc);
        count_launch(ctx);
        // per column: Hessenberg (column-major (m+1) x m), Givens, g
        std::vector<std::vector<cd>> H(nrhs, std::vector<cd>(size_t(m + 1) * m, 0.0)), g(nrhs, std::vector<cd>(m + 1, 0.0));
        std::vector<std::vector<double>> cs(nrhs, std::vector<double>(m, 0.0));
        std::vector<std::vector<cd>> sn(nrhs, std::vector<cd>(m, 0.0));
        std::vector<int> kcol(nrhs, 0);
        for (int c = 0; c < nrhs; c++) g[c][0] = beta[c];
        int j = 0;
        for (; j < m && total < max_iters; j++, total++) {
            if ((rc = precond_apply_fp32(ctx, V + int64_t(j) * n, ldc, nrhs, U))) return rc;
            if ((rc = cuda_check(ctx, cudaMemcpy2DAsync(Zb + int64_t(j) * n, sizeof(double2) * ldz, U,
                                                        sizeof(double2) * n, sizeof(double2) * n, nrhs,
                                                        cudaMemcpyDeviceToDevice, st), "gmres z")))
                return rc;
            // W = Z U, orthogonalised against V (two classical Gram-Schmidt passes), its norms
            auto arnoldi = [&](bool df) -> int {
                int r2 = matvec_z64(ctx, U, nrhs, W, df);
                if (r2) return r2;
                for (int pass = 0; pass < 2; pass++) {
                    double2* hp = dh + size_t(pass) * nrhs * (m + 1);
                    k_gs_dots<<<dim3(j + 1, nrhs), 256, 0, st>>>(n, V, ldc, W, hp, m + 1);
                    k_gs_axpy<<<g1, 256, 0, st>>>(n, nrhs, j + 1, V, ldc, hp, m + 1, W);
                    count_launch(ctx, 2);
                }
                k_norm2_cols<<<nrhs, 256, 0, st>>>(n, W, dnr);
                count_launch(ctx);
                r2 = cuda_check(ctx, cudaMemcpyAsync(hh.data(), dh, sizeof(double2) * hh.size(), cudaMemcpyDeviceToHost,
                                                     st), "gmres h");
                if (!r2)
                    r2 = cuda_check(ctx, cudaMemcpyAsync(hnorm.data(), dnr, sizeof(double) * nrhs,
                                                         cudaMemcpyDeviceToHost, st), "gmres hn");
                return r2;
            };
            if ((rc = arnoldi(use_df))) return rc;
            DeviceStatus hs;
            if ((rc = trsv_check(ctx, &hs))) return rc;   // (waits for the stream)
            if (use_df && hs.df_range) {   // an operand outside the double-float range: FP64 from here on
                use_df = false;
                if ((rc = arnoldi(false)) || (rc = trsv_check(ctx))) return rc;
            }
            bool all_done = true;
            for (int c = 0; c < nrhs; c++) {
                hscale[c] = 0.0;
                if (done[c]) continue;
                std::vector<cd>& Hc = H[c];
                cd* col = &Hc[size_t(j) * (m + 1)];
                for (int i = 0; i <= j; i++) {
                    const double2 a = hh[size_t(c) * (m + 1) + i], b = hh[size_t(nrhs + c) * (m + 1) + i];
                    col[i] = cd(a.x + b.x, a.y + b.y);
                }
                const double hn = std::sqrt(hnorm[c]);
                col[j + 1] = hn;
                for (int i = 0; i < j; i++) {   // previous rotations
                    const cd t = cs[c][i] * col[i] + sn[c][i] * col[i + 1];
                    col[i + 1] = -std::conj(sn[c][i]) * col[i] + cs[c][i] * col[i + 1];
                    col[i] = t;
                }
                const double a = std::abs(col[j]), bb = std::abs(col[j + 1]);
                const double den = std::sqrt(a * a + bb * bb);
                if (den > 0) {
                    cs[c][j] = a / den;
                    sn[c][j] = a > 0 ? (col[j] / a) * std::conj(col[j + 1]) / den : cd(1.0, 0.0);
                } else {
                    cs[c][j] = 1.0;
                    sn[c][j] = 0.0;
                }
                col[j] = cs[c][j] * col[j] + sn[c][j] * col[j + 1];
                col[j + 1] = 0.0;
                g[c][j + 1] = -std::conj(sn[c][j]) * g[c][j];
                g[c][j] = cs[c][j] * g[c][j];
                kcol[c] = j + 1;
                const double est = std::abs(g[c][j + 1]) / bnorm[c];
                if (!(est > 0.1 * tol) || !(hn > 1e-300 * beta[c])) {
                    done[c] = true;
                } else {
                    hscale[c] = 1.0 / hn;
                    all_done = false;
                }
            }
            if (all_done) {
                j++;
                total++;
                break;
            }
            if ((rc = cuda_check(ctx, cudaMemcpyAsync(dsc, hscale.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice,
                                                      st), "gmres scale")))
                return rc;
            k_scale_cols<<<g1, 256, 0, st>>>(n, nrhs, W, n, dsc, V + int64_t(j + 1) * n, ldc);
            count_launch(ctx);
        }
        // y = R^{-1} g per column, x += Z y with the stored z_i = M^{-1} v_i (flexible GMRES:
        // applying the complex64 preconditioner once more to V y would add its rounding,
        // which near kappa * eps32 = 1 stalls the residual above the target)
        std::fill(hy.begin(), hy.end(), double2{0.0, 0.0});
        int kmax = 0;
        for (int c = 0; c < nrhs; c++) {
            const int k = kcol[c];
            if (!active[c] || k == 0) continue;
            kmax = std::max(kmax, k);
            std::vector<cd> y(k);
            for (int i = k - 1; i >= 0; i--) {
                cd s = g[c][i];
                for (int q = i + 1; q < k; q++) s -= H[c][size_t(q) * (m + 1) + i] * y[q];
                y[i] = s / H[c][size_t(i) * (m + 1) + i];
            }
            for (int i = 0; i < k; i++) hy[size_t(c) * (m + 1) + i] = double2{y[i].real(), y[i].imag()};
        }
        if (kmax == 0) break;
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(dy, hy.data(), sizeof(double2) * hy.size(), cudaMemcpyHostToDevice, st),
                             "gmres y")))
            return rc;
        k_combine<<<g1, 256, 0, st>>>(n, nrhs, kmax, Zb, ldz, dy, m + 1, D);
        k_add_to<<<g1, 256, 0, st>>>(cnt, D, X);
        count_launch(ctx, 2);
        // true residual
        if ((rc = matvec_fp64(ctx, X, nrhs, W))) return rc;
        k_sub<<<g1, 256, 0, st>>>(cnt, B, W, R);
        count_launch(ctx);
        if ((rc = colnorms(R))) return rc;
    }
    *iters_out = total;
    *rel_out = rel;
    return cuda_check(ctx, cudaGetLastError(), "gmres");
}

}  // namespace frico
