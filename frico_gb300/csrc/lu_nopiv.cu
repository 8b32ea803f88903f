// Blocked complex LU without row interchanges, for the mixed-precision path.
//
// The complex64 factors of the mixed path only precondition an iterative
// refinement whose residual is computed against the FP64 Z, so the pivoting
// strategy affects the number of refinement sweeps, not the accuracy of the
// result. EFIE impedance matrices (RWG, Dunavant quadrature) factor stably
// without interchanges (growth 2.3 on the 7680-unknown sphere), and dropping
// the pivot search removes the n sequential cluster-wide argmax steps of the
// partial-pivoting panel. The caller falls back to partial pivoting when a
// pivot is zero / not finite (info != 0) or the refinement does not converge.
//
// Per block column k0 (width nb = 128):
//   k_diag_lu      one CTA: LU of the nb x nb diagonal block in shared memory,
//                  then U11^{-1} (triangular inverse) into a workspace
//   k_trsm_right   L21 = A21 U11^{-1}, 64 rows per CTA
//   k_trsm_lower_unit (lu.cu)   U12 = L11^{-1} A12
//   trailing update A22 -= L21 U12 (tensor cores when available)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "common.cuh"

namespace frico {

static const int kNP = 128;   // block width of the no-pivot LU

template <typename C> __device__ __forceinline__ bool cfinite(C a) { return isfinite(a.x) && isfinite(a.y); }

// In-place inverse of the upper triangle of the jb x jb column-major block a
// (entries below the diagonal are neither read nor written). With unit = 1 the
// diagonal is taken as 1. Column j of the inverse needs only columns < j:
//   X[j][j] = 1/U[j][j],  X[i][j] = -(sum_{k=i}^{j-1} X[i][k] U[k][j]) X[j][j]
// 512 threads: thread (i, g) sums the k = g mod 4 terms of row i.
template <typename C>
__device__ void upper_inverse_inplace(C* a, int jb, bool unit, C (*red)[kNP]) {
    using R = decltype(a[0].x);
    const int i = threadIdx.x & (kNP - 1), g = threadIdx.x >> 7;
    for (int j = 0; j < jb; j++) {
        const C xjj = unit ? cmake(R(1), R(0)) : cdiv(cmake(R(1), R(0)), a[j * jb + j]);
        C s = cmake(R(0), R(0));
        if (i < j)
            for (int k = i + g; k < j; k += 4) {
                const C xik = (k == i) ? (unit ? cmake(R(1), R(0)) : a[i * jb + i]) : a[k * jb + i];
                s = cadd(s, cmul(xik, a[j * jb + k]));
            }
        red[g][i] = s;
        __syncthreads();
        if (g == 0) {
            if (i < j) {
                C t = cadd(cadd(red[0][i], red[1][i]), cadd(red[2][i], red[3][i]));
                a[j * jb + i] = cmul(cmake(-t.x, -t.y), xjj);
            } else if (i == j && !unit) {
                a[j * jb + j] = xjj;
            }
        }
        __syncthreads();
    }
}

// LU (no interchanges) of the jb x jb diagonal block at (k0, k0), written back
// in place; then U11^{-1} (upper) to Uinv and L11^{-1} (unit lower) to Linv,
// both jb x jb column-major with leading dimension jb. 512 threads: thread
// (row r, column group g) updates columns c+1+g, c+5+g, ... of row r.
template <typename C>
__global__ void __launch_bounds__(512) k_diag_lu(C* A, int64_t lda, int k0, int jb, C* Uinv, C* Linv,
                                                DeviceStatus* st) {
    using R = decltype(A[0].x);
    extern __shared__ __align__(16) unsigned char smraw[];
    C* a = (C*)smraw;   // a[c * jb + r]
    __shared__ C red[4][kNP];
    for (int idx = threadIdx.x; idx < jb * jb; idx += blockDim.x) {
        int r = idx % jb, c = idx / jb;
        a[idx] = A[int64_t(k0 + c) * lda + k0 + r];
    }
    __syncthreads();
    const int r = threadIdx.x & (kNP - 1), g = threadIdx.x >> 7;
    for (int c = 0; c < jb; c++) {
        const C p = a[c * jb + c];
        const bool bad = (p.x == R(0) && p.y == R(0)) || !cfinite(p);
        const C inv = bad ? cmake(R(0), R(0)) : cdiv(cmake(R(1), R(0)), p);
        if (bad && threadIdx.x == 0) atomicCAS(&st->info, 0, k0 + c + 1);
        if (g == 0 && r > c && r < jb) a[c * jb + r] = cmul(a[c * jb + r], inv);
        __syncthreads();
        if (r > c && r < jb) {
            const C l = a[c * jb + r];
            for (int cc = c + 1 + g; cc < jb; cc += 4) a[cc * jb + r] = cfms(a[cc * jb + r], l, a[cc * jb + c]);
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < jb * jb; idx += blockDim.x) {
        int rr = idx % jb, c = idx / jb;
        A[int64_t(k0 + c) * lda + k0 + rr] = a[idx];
    }
    upper_inverse_inplace(a, jb, false, red);
    for (int idx = threadIdx.x; idx < jb * jb; idx += blockDim.x) {
        int rr = idx % jb, c = idx / jb;
        Uinv[idx] = rr <= c ? a[idx] : cmake(R(0), R(0));
    }
    __syncthreads();
    // L^{-1} = ((L^T)^{-1})^T: reload the factored block transposed, so that
    // L^T sits in the upper triangle, and invert it with unit diagonal.
    for (int idx = threadIdx.x; idx < jb * jb; idx += blockDim.x) {
        int rr = idx % jb, c = idx / jb;               // global (row rr, col c)
        a[rr * jb + c] = A[int64_t(k0 + c) * lda + k0 + rr];
    }
    __syncthreads();
    upper_inverse_inplace(a, jb, true, red);
    for (int idx = threadIdx.x; idx < jb * jb; idx += blockDim.x) {
        int rr = idx % jb, c = idx / jb;               // Linv (row rr, col c) = Tinv (row c, col rr)
        Linv[idx] = rr > c ? a[rr * jb + c] : (rr == c ? cmake(R(1), R(0)) : cmake(R(0), R(0)));
    }
}

// A[r0 + 64*blockIdx.x ..., k0:k0+jb] <- that block times U11^{-1}.
// Thread (row, column group of 32): 32 outputs accumulated in registers.
template <typename C>
__global__ void __launch_bounds__(256) k_trsm_right(C* A, int64_t lda, int r0, int r1, int k0, int jb,
                                                   const C* __restrict__ Uinv) {
    using R = decltype(A[0].x);
    extern __shared__ __align__(16) unsigned char smraw[];
    C* u = (C*)smraw;            // Uinv[c * jb + r]
    C* blk = u + jb * jb;        // blk[q * 64 + row]
    const int rb = r0 + blockIdx.x * 64;
    const int nr = min(64, r1 - rb);
    for (int idx = threadIdx.x; idx < jb * jb; idx += blockDim.x) u[idx] = Uinv[idx];
    for (int idx = threadIdx.x; idx < 64 * jb; idx += blockDim.x) {
        int row = idx & 63, q = idx >> 6;
        blk[q * 64 + row] = row < nr ? A[int64_t(k0 + q) * lda + rb + row] : cmake(R(0), R(0));
    }
    __syncthreads();
    const int row = threadIdx.x & 63, cg = threadIdx.x >> 6;   // 4 groups
    for (int c0 = cg * 32; c0 < jb; c0 += 128) {
        C acc[32];
#pragma unroll
        for (int j = 0; j < 32; j++) acc[j] = cmake(R(0), R(0));
        for (int q = 0; q < jb; q++) {
            const C x = blk[q * 64 + row];
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const C w = u[(c0 + j) * jb + q];   // broadcast
                acc[j].x += x.x * w.x - x.y * w.y;
                acc[j].y += x.x * w.y + x.y * w.x;
            }
        }
        if (row < nr)
#pragma unroll
            for (int j = 0; j < 32; j++)
                if (c0 + j < jb) A[int64_t(k0 + c0 + j) * lda + rb + row] = acc[j];
    }
}

// ------------------------------------------------------------------ host side
template <typename C> __global__ void k_ipiv_identity(int n, int32_t* ipiv, int32_t* perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        ipiv[i] = i + 1;
        perm[i] = i;
    }
}

int trsm_lower_unit_f32(frico_gpu_ctx* ctx, float2* A, int64_t lda, int k0, int jb, int cb, int ce);  // lu.cu

int lu_factor_nopiv_fp32(frico_gpu_ctx* ctx) {
    using C = float2;
    C* A = (C*)ctx->z32.p;
    const int n = int(ctx->n);
    const int64_t lda = ctx->n;
    cudaStream_t st = ctx->stream;
    int rc;
    if ((rc = ensure(ctx, ctx->ipiv, sizeof(int32_t) * n))) return rc;
    if ((rc = ensure(ctx, ctx->perm, sizeof(int32_t) * n))) return rc;
    if ((rc = ensure(ctx, ctx->status, sizeof(DeviceStatus)))) return rc;
    if ((rc = ensure(ctx, ctx->panel_ws, sizeof(C) * 2 * kNP * kNP + 256))) return rc;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(DeviceStatus), st), "status"))) return rc;
    DeviceStatus* dst = (DeviceStatus*)ctx->status.p;
    C* Uinv = (C*)ctx->panel_ws.p;
    C* Linv = Uinv + kNP * kNP;
    const size_t diag_smem = sizeof(C) * kNP * kNP;
    const size_t right_smem = sizeof(C) * (kNP * kNP + 64 * kNP);
    static bool attrs = false;
    if (!attrs) {
        if ((rc = cuda_check(ctx, cudaFuncSetAttribute(k_diag_lu<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      int(diag_smem)), "diag smem")))
            return rc;
        if ((rc = cuda_check(ctx, cudaFuncSetAttribute(k_trsm_right<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      int(right_smem)), "trsm_right smem")))
            return rc;
        attrs = true;
    }
    const bool tc = ctx->opt.gemm_engine != FRICO_GEMM_SIMT && gemm_tc_available(ctx);
    if (ctx->opt.gemm_engine == FRICO_GEMM_TC && !tc)
        return set_err(ctx, FRICO_GPU_EINVAL, "tensor-core GEMM engine not available on this device");
    k_ipiv_identity<C><<<(n + 255) / 256, 256, 0, st>>>(n, (int32_t*)ctx->ipiv.p, (int32_t*)ctx->perm.p);
    count_launch(ctx);
    for (int k0 = 0; k0 < n; k0 += kNP) {
        const int jb = std::min(kNP, n - k0);
        k_diag_lu<C><<<1, 512, sizeof(C) * jb * jb, st>>>(A, lda, k0, jb, Uinv, Linv, dst);
        count_launch(ctx);
        const int rest = n - k0 - jb;
        if (rest > 0) {
            C* A21 = A + int64_t(k0) * lda + k0 + jb;
            C* A12 = A + int64_t(k0 + jb) * lda + k0;
            if (tc) {
                // L21 = A21 U11^{-1},  U12 = L11^{-1} A12 on the tensor cores (overwrite mode)
                if ((rc = gemm_update_tc(ctx, A21, lda, A21, lda, Uinv, jb, rest, jb, jb, nullptr, 0))) return rc;
                if ((rc = gemm_update_tc(ctx, A12, lda, Linv, jb, A12, lda, jb, rest, jb, nullptr, 0))) return rc;
            } else {
                k_trsm_right<C><<<(rest + 63) / 64, 256, sizeof(C) * (jb * jb + 64 * jb), st>>>(A, lda, k0 + jb, n,
                                                                                                k0, jb, Uinv);
                count_launch(ctx);
                if ((rc = trsm_lower_unit_f32(ctx, A, lda, k0, jb, k0 + jb, n))) return rc;
            }
            C* Cm = A + int64_t(k0 + jb) * lda + k0 + jb;
            const C* Lm = A + int64_t(k0) * lda + k0 + jb;
            const C* Um = A + int64_t(k0 + jb) * lda + k0;
            cudaEvent_t* ev = prof_event_pair(ctx);
            if (ev) {
                ctx->stats.gemm_flops += 8.0 * double(rest) * double(rest) * double(jb);
                ctx->stats.gemm_bytes += sizeof(C) * (2.0 * double(rest) * double(rest) + 2.0 * double(rest) * jb);
            }
            if (tc) {
                if ((rc = gemm_update_tc(ctx, Cm, lda, Lm, lda, Um, lda, rest, rest, jb, ev))) return rc;
            } else {
                if (ev) cudaEventRecord(ev[0], st);
                if ((rc = gemm_update_simt32(ctx, Cm, lda, Lm, lda, Um, lda, rest, rest, jb))) return rc;
                if (ev) cudaEventRecord(ev[1], st);
            }
        }
        if ((rc = cuda_check(ctx, cudaGetLastError(), "nopiv lu step"))) return rc;
    }
    prof_event_collect(ctx);
    DeviceStatus hs;
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, st), "status")))
        return rc;
    if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "nopiv lu sync"))) return rc;
    if (hs.err == FRICO_DEV_ERR_TIMEOUT) return set_err(ctx, FRICO_GPU_ETIMEOUT, "tensor-core GEMM wait timed out");
    ctx->info = hs.info;
    if (hs.info != 0) return FRICO_GPU_OK;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(DeviceStatus), st), "status reset")))
        return rc;
    return trsv_prepare_fp32(ctx);
}

}  // namespace frico
