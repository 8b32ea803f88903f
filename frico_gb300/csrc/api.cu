// C-ABI entry points (include/frico_gpu.h). Argument checking, context state,
// host<->device copies and the host-side arithmetic on the few values that
// come back (port values, gain, RCS) live here; every O(N^2) / O(N^3) stage is
// a kernel in fill.cu, lu.cu or fields.cu.
#include <cuda_runtime.h>

#include <mutex>
#include <set>

#include <algorithm>
#include <climits>
#include <cmath>
#include <complex>
#include <cstring>
#include <new>

#include "common.cuh"
#include "frico_gpu_debug.h"

namespace frico {

int set_err(frico_gpu_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

int cuda_check(frico_gpu_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return FRICO_GPU_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return set_err(ctx, e == cudaErrorMemoryAllocation ? FRICO_GPU_ENOMEM : FRICO_GPU_ECUDA, m);
}

int ensure(frico_gpu_ctx* ctx, DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return FRICO_GPU_OK;
    if (b.p) {
        cudaStreamSynchronize(ctx->stream);
        if (ctx->stream2) cudaStreamSynchronize(ctx->stream2);
        cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return cuda_check(ctx, e, "cudaMalloc");
    }
    b.bytes = bytes;
    return FRICO_GPU_OK;
}

void release(DevBuf& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

static frico_gpu_options default_options() {
    frico_gpu_options o;
    std::memset(&o, 0, sizeof o);
    o.degree = 1;
    o.precision = FRICO_PREC_FP64;
    o.h_phase_mode = FRICO_HPHASE_COMPAT;
    o.max_refine_iters = 30;
    o.refine_tol = 1e-12;
    o.Z0 = 50.0;
    return o;
}

static int check_options(frico_gpu_ctx* ctx, const frico_gpu_options* o) {
    if (o->degree < 0 || o->degree > 20) return set_err(ctx, FRICO_GPU_EINVAL, "Dunavant quadrature: degree too high");
    if (o->precision != FRICO_PREC_FP64 && o->precision != FRICO_PREC_MIXED)
        return set_err(ctx, FRICO_GPU_EINVAL, "unknown precision");
    if (o->h_phase_mode != FRICO_HPHASE_COMPAT && o->h_phase_mode != FRICO_HPHASE_PHYSICAL)
        return set_err(ctx, FRICO_GPU_EINVAL, "unknown h_phase_mode");
    if (o->gemm_engine < FRICO_GEMM_AUTO || o->gemm_engine > FRICO_GEMM_TC_F16)
        return set_err(ctx, FRICO_GPU_EINVAL, "unknown gemm_engine");
    if (o->pivoting < FRICO_PIVOT_AUTO || o->pivoting > FRICO_PIVOT_NONE)
        return set_err(ctx, FRICO_GPU_EINVAL, "unknown pivoting");
    if (o->refine_mode != FRICO_REFINE_AUTO && o->refine_mode != FRICO_REFINE_CLASSIC)
        return set_err(ctx, FRICO_GPU_EINVAL, "unknown refine_mode");
    if (o->residual_mode != FRICO_RESIDUAL_AUTO && o->residual_mode != FRICO_RESIDUAL_FP64)
        return set_err(ctx, FRICO_GPU_EINVAL, "unknown residual_mode");
    if (o->fields_engine < FRICO_FIELDS_AUTO || o->fields_engine > FRICO_FIELDS_GEMM)
        return set_err(ctx, FRICO_GPU_EINVAL, "unknown fields_engine");
    return FRICO_GPU_OK;
}

static int use_device(frico_gpu_ctx* ctx) { return cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"); }

}  // namespace frico

using namespace frico;

namespace frico {
int device_once(frico_gpu_ctx* ctx, OnceKey key, int (*init)(frico_gpu_ctx*)) {
    static std::mutex mu;
    static std::set<std::pair<int, int>> done;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({ctx->device, int(key)})) return FRICO_GPU_OK;
    const int rc = init(ctx);
    if (rc == FRICO_GPU_OK) done.insert({ctx->device, int(key)});
    return rc;
}
}  // namespace frico

#define FRICO_CTX_CHECK(ctx)                                 \
    do {                                                     \
        if (!(ctx)) return FRICO_GPU_EINVAL;                 \
        int _rc = use_device(ctx);                           \
        if (_rc) return _rc;                                 \
    } while (0)

extern "C" int frico_gpu_ctx_create(frico_gpu_ctx** out, int device, const frico_gpu_options* opt) {
    if (!out) return FRICO_GPU_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return FRICO_GPU_ECUDA;
    }
    if (device < 0 || device >= ndev) return FRICO_GPU_EINVAL;
    frico_gpu_ctx* ctx = new (std::nothrow) frico_gpu_ctx();
    if (!ctx) return FRICO_GPU_ENOMEM;
    ctx->device = device;
    ctx->opt = opt ? *opt : default_options();
    if (ctx->opt.Z0 == 0.0) ctx->opt.Z0 = 50.0;
    int rc = check_options(ctx, &ctx->opt);
    if (!rc) rc = use_device(ctx);
    if (!rc) rc = cuda_check(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream");
    if (!rc) rc = cuda_check(ctx, cudaEventCreate(&ctx->ev0), "event");
    if (!rc) rc = cuda_check(ctx, cudaEventCreate(&ctx->ev1), "event");
    if (rc) {
        frico_gpu_ctx_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_ctx_destroy(frico_gpu_ctx* ctx) {
    if (!ctx) return FRICO_GPU_EINVAL;
    destroy_lanes(ctx);
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    DevBuf* bufs[] = {&ctx->xyz,     &ctx->tri,      &ctx->trigeo,   &ctx->qp,        &ctx->qps,     &ctx->rwg_itm,
                      &ctx->rwg_itp, &ctx->rwg_len,  &ctx->rwg_am,   &ctx->rwg_ap,    &ctx->rwg_vm,  &ctx->rwg_vp,
                      &ctx->rwg_itf, &ctx->tri_bf,   &ctx->tri_new,  &ctx->tri_old,   &ctx->gtab,     &ctx->smom,      &ctx->basis_aux, &ctx->z64,
                      &ctx->z32,     &ctx->z64_keep, &ctx->res64,    &ctx->ipiv,     &ctx->perm,      &ctx->panel_ws, &ctx->status,
                      &ctx->rhs,     &ctx->sol,      &ctx->rwork,    &ctx->rwork32,   &ctx->dwork32, &ctx->norms,
                      &ctx->tri_aj,  &ctx->tri_adivj, &ctx->tri_j,   &ctx->fld_pts,   &ctx->fld_part, &ctx->fld_out,
                      &ctx->dinv,    &ctx->trsv_flags, &ctx->tc_ws,   &ctx->lut,       &ctx->dinv_t,
                      &ctx->adj_ws,  &ctx->adj_tab, &ctx->mlump,     &ctx->mfld,     &ctx->gm_ws,
                      &ctx->dinv128, &ctx->trsv_x, &ctx->ffws};
    for (DevBuf* b : bufs) release(*b);
    for (cudaEvent_t e : ctx->prof_events) cudaEventDestroy(e);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream2) cudaStreamSynchronize(ctx->stream2);
    if (ctx->lu_graph.exec) cudaGraphExecDestroy(ctx->lu_graph.exec);
    for (cudaEvent_t e : ctx->la_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_set_options(frico_gpu_ctx* ctx, const frico_gpu_options* opt) {
    if (!ctx || !opt) return FRICO_GPU_EINVAL;
    int rc = check_options(ctx, opt);
    if (rc) return rc;
    bool refill = opt->degree != ctx->opt.degree || opt->approx != ctx->opt.approx ||
                  opt->force_symmetry != ctx->opt.force_symmetry || opt->precision != ctx->opt.precision ||
                  opt->pivoting != ctx->opt.pivoting || opt->gemm_engine != ctx->opt.gemm_engine;
    ctx->opt = *opt;
    if (ctx->opt.Z0 == 0.0) ctx->opt.Z0 = 50.0;
    if (refill) {
        ctx->z_valid = false;
        ctx->factored = false;
        ctx->solved = false;
    }
    return FRICO_GPU_OK;
}

extern "C" const char* frico_gpu_last_error(frico_gpu_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

extern "C" int frico_gpu_get_stream(frico_gpu_ctx* ctx, void** stream) {
    if (!ctx || !stream) return FRICO_GPU_EINVAL;
    *stream = (void*)ctx->stream;
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_set_mesh(frico_gpu_ctx* ctx, int64_t nv, const double* xyz, int64_t nt, const int64_t* tri,
                                  int64_t n, const frico_rwg* rwg) {
    FRICO_CTX_CHECK(ctx);
    if (nv <= 0 || nt <= 0 || n <= 0 || !xyz || !tri || !rwg)
        return set_err(ctx, FRICO_GPU_EINVAL, "set_mesh: empty mesh or null pointer");
    if (nt > INT32_MAX || n > INT32_MAX) return set_err(ctx, FRICO_GPU_EINVAL, "set_mesh: mesh too large");
    for (int64_t i = 0; i < 3 * nt; i++)
        if (tri[i] < 0 || tri[i] >= nv) return set_err(ctx, FRICO_GPU_EINVAL, "set_mesh: vertex index out of range");
    std::vector<int32_t> itm(n), itp(n), itf(n);
    std::vector<double> len(n), am(n), ap(n), vm(3 * n), vp(3 * n);
    std::vector<int32_t> tri_bf(3 * nt, 0);
    std::vector<int> fill_cnt(nt, 0);
    for (int64_t i = 0; i < n; i++) {
        const frico_rwg& b = rwg[i];
        if (b.matrix_index != i) return set_err(ctx, FRICO_GPU_EINVAL, "set_mesh: rwg[i].matrix_index must equal i");
        if (b.itminus < 0 || b.itminus >= nt || b.itplus < 0 || b.itplus >= nt || b.itminus == b.itplus)
            return set_err(ctx, FRICO_GPU_EINVAL, "set_mesh: rwg triangle index out of range");
        if (!(b.Aminus > 0) || !(b.Aplus > 0)) return set_err(ctx, FRICO_GPU_EINVAL, "set_mesh: non-positive triangle area");
        itm[i] = int32_t(b.itminus);
        itp[i] = int32_t(b.itplus);
        itf[i] = b.has_interface ? b.interface_tag : INT32_MIN;
        len[i] = b.length;
        am[i] = b.Aminus;
        ap[i] = b.Aplus;
        for (int d = 0; d < 3; d++) {
            vm[3 * i + d] = b.pminus[d];
            vp[3 * i + d] = b.pplus[d];
        }
        // per-triangle slots in increasing matrix index (run_context order)
        for (int side = 0; side < 2; side++) {
            int64_t t = side ? b.itplus : b.itminus;
            if (fill_cnt[t] >= 3) return set_err(ctx, FRICO_GPU_EMESH, "set_mesh: triangle with more than 3 RWG edges");
            tri_bf[3 * t + fill_cnt[t]++] = side ? int32_t(i + 1) : -int32_t(i + 1);
        }
    }
    std::vector<int32_t> tri_new(nt, -1), tri_old(nt);
    int32_t next = 0;
    for (int64_t i = 0; i < n; i++)
        for (const int32_t t : {itm[i], itp[i]})
            if (tri_new[t] < 0) {
                tri_new[t] = next;
                tri_old[next++] = t;
            }
    for (int64_t t = 0; t < nt; t++)   // triangles without an RWG edge
        if (tri_new[t] < 0) {
            tri_new[t] = next;
            tri_old[next++] = int32_t(t);
        }
    int rc;
    // all arrays through one pinned staging buffer: asynchronous copies on the context's
    // stream, then one synchronisation (the data is on the device when this returns)
    struct Up {
        DevBuf* b;
        const void* src;
        size_t bytes;
    };
    const Up ups[] = {{&ctx->xyz, xyz, sizeof(double) * 3 * nv},
                      {&ctx->tri, tri, sizeof(int64_t) * 3 * nt},
                      {&ctx->rwg_itm, itm.data(), sizeof(int32_t) * n},
                      {&ctx->rwg_itp, itp.data(), sizeof(int32_t) * n},
                      {&ctx->rwg_itf, itf.data(), sizeof(int32_t) * n},
                      {&ctx->rwg_len, len.data(), sizeof(double) * n},
                      {&ctx->rwg_am, am.data(), sizeof(double) * n},
                      {&ctx->rwg_ap, ap.data(), sizeof(double) * n},
                      {&ctx->rwg_vm, vm.data(), sizeof(double) * 3 * n},
                      {&ctx->rwg_vp, vp.data(), sizeof(double) * 3 * n},
                      {&ctx->tri_bf, tri_bf.data(), sizeof(int32_t) * 3 * nt},
                      {&ctx->tri_new, tri_new.data(), sizeof(int32_t) * nt},
                      {&ctx->tri_old, tri_old.data(), sizeof(int32_t) * nt}};
    size_t total = 0;
    for (const Up& u : ups) total += (u.bytes + 255) & ~size_t(255);
    // the previous upload from the staging buffer has finished: its call synchronised
    if (total > ctx->h_stage_bytes) {
        if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
        ctx->h_stage = nullptr;
        ctx->h_stage_bytes = 0;
        if ((rc = cuda_check(ctx, cudaHostAlloc(&ctx->h_stage, total, cudaHostAllocDefault), "pinned staging")))
            return rc;
        ctx->h_stage_bytes = total;
    }
    size_t off = 0;
    for (const Up& u : ups) {
        if ((rc = ensure(ctx, *u.b, u.bytes))) return rc;
        char* h = (char*)ctx->h_stage + off;
        std::memcpy(h, u.src, u.bytes);
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(u.b->p, h, u.bytes, cudaMemcpyHostToDevice, ctx->stream), "upload")))
            return rc;
        off += (u.bytes + 255) & ~size_t(255);
    }
    if ((rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "upload sync"))) return rc;
    ctx->nv = nv;
    ctx->nt = nt;
    ctx->n = n;
    ctx->h_rwg.assign(rwg, rwg + n);
    ctx->h_xyz.assign(xyz, xyz + 3 * nv);
    ctx->h_tri.assign(tri, tri + 3 * nt);
    ctx->mesh_gen++;
    ctx->geo_degree = -1;
    ctx->z_valid = ctx->factored = ctx->solved = false;
    ctx->z64_keep_valid = false;
    ctx->lumped_col = -1;
    ctx->nrhs = 0;
    ctx->stats = frico_gpu_stats{};
    ctx->stats.n = n;
    ctx->stats.ntri = nt;
    return build_quadrature(ctx);
}

extern "C" int frico_gpu_fill(frico_gpu_ctx* ctx, double freq, frico_c128* Z_out, int64_t ldz) {
    FRICO_CTX_CHECK(ctx);
    if (ctx->n <= 0) return set_err(ctx, FRICO_GPU_ESTATE, "fill: no mesh");
    if (!(freq > 0) || !std::isfinite(freq)) return set_err(ctx, FRICO_GPU_EINVAL, "fill: frequency must be > 0");
    if (Z_out && ldz < ctx->n) return set_err(ctx, FRICO_GPU_EINVAL, "fill: ldz < n");
    int rc;
    {
        StageTimer tm(ctx, &ctx->stats.fill_ms);
        rc = fill_matrix(ctx, freq);
    }
    if (rc) return rc;
    ctx->z_valid = true;
    ctx->z32_stale = false;
    ctx->z64_keep_valid = false;
    ctx->factored = ctx->solved = false;
    ctx->lumped_col = -1;
    if (Z_out) {
        rc = cuda_check(ctx, cudaMemcpy2DAsync(Z_out, sizeof(frico_c128) * ldz, ctx->z64.p, sizeof(double2) * ctx->n,
                                               sizeof(double2) * ctx->n, ctx->n, cudaMemcpyDeviceToHost, ctx->stream),
                        "copy Z");
        if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "fill sync");
    }
    return rc;
}

extern "C" int frico_gpu_set_matrix(frico_gpu_ctx* ctx, double freq, const frico_c128* Z, int64_t ldz) {
    FRICO_CTX_CHECK(ctx);
    if (ctx->n <= 0) return set_err(ctx, FRICO_GPU_ESTATE, "set_matrix: no mesh");
    if (!Z || ldz < ctx->n) return set_err(ctx, FRICO_GPU_EINVAL, "set_matrix: null Z or ldz < n");
    if (!(freq > 0) || !std::isfinite(freq)) return set_err(ctx, FRICO_GPU_EINVAL, "set_matrix: frequency must be > 0");
    const int64_t n = ctx->n;
    int rc = ensure(ctx, ctx->z64, sizeof(double2) * size_t(n) * size_t(n));
    if (!rc)
        rc = cuda_check(ctx, cudaMemcpy2DAsync(ctx->z64.p, sizeof(double2) * n, Z, sizeof(frico_c128) * ldz,
                                               sizeof(double2) * n, n, cudaMemcpyHostToDevice, ctx->stream),
                        "upload Z");
    // solve_symmetric (zsytrf, uplo = 'U') reads only the upper triangle of its argument
    if (!rc && (ctx->opt.approx || ctx->opt.force_symmetry)) rc = mirror_upper(ctx);
    if (!rc && ctx->opt.precision == FRICO_PREC_MIXED) rc = z64_to_z32(ctx);
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "set_matrix sync");
    if (rc) return rc;
    ctx->freq = freq;
    ctx->z_valid = true;
    ctx->z32_stale = false;
    ctx->z64_keep_valid = false;
    ctx->z_df = false;   // an FP64 Z as given: nothing to reassemble before an FP64 fallback
    ctx->factored = ctx->solved = false;
    ctx->lumped_col = -1;
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_set_nrhs(frico_gpu_ctx* ctx, int32_t nrhs) {
    FRICO_CTX_CHECK(ctx);
    if (ctx->n <= 0) return set_err(ctx, FRICO_GPU_ESTATE, "set_nrhs: no mesh");
    if (nrhs <= 0 || nrhs > 4096) return set_err(ctx, FRICO_GPU_EINVAL, "set_nrhs: nrhs out of range");
    int rc = ensure(ctx, ctx->rhs, sizeof(double2) * ctx->n * nrhs);
    if (!rc) rc = cuda_check(ctx, cudaMemsetAsync(ctx->rhs.p, 0, sizeof(double2) * ctx->n * nrhs, ctx->stream), "memset");
    if (rc) return rc;
    ctx->nrhs = nrhs;
    ctx->solved = false;
    ctx->lumped_col = -1;
    return FRICO_GPU_OK;
}

static int check_col(frico_gpu_ctx* ctx, int32_t col) {
    if (ctx->nrhs <= 0) return set_err(ctx, FRICO_GPU_ESTATE, "no right-hand sides (call set_nrhs)");
    if (col < 0 || col >= ctx->nrhs) return set_err(ctx, FRICO_GPU_EINVAL, "rhs column out of range");
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_rhs_delta_gap(frico_gpu_ctx* ctx, double freq, int32_t col, int32_t n_itf,
                                       const int32_t* itf_tags, frico_c128 V0, const double* signs) {
    FRICO_CTX_CHECK(ctx);
    int rc = check_col(ctx, col);
    if (rc) return rc;
    if (!(freq > 0)) return set_err(ctx, FRICO_GPU_EINVAL, "rhs: frequency must be > 0");
    if (n_itf < 0 || (n_itf > 0 && !itf_tags)) return set_err(ctx, FRICO_GPU_EINVAL, "rhs: bad interface list");
    StageTimer tm(ctx, &ctx->stats.rhs_ms);
    ctx->solved = false;
    return rhs_delta_gap(ctx, freq, col, n_itf, itf_tags, make_double2(V0.re, V0.im), signs);
}

extern "C" int frico_gpu_rhs_plane_wave(frico_gpu_ctx* ctx, double freq, int32_t col, double theta, double phi,
                                        frico_c128 Etheta, frico_c128 Ephi) {
    FRICO_CTX_CHECK(ctx);
    int rc = check_col(ctx, col);
    if (rc) return rc;
    if (!(freq > 0)) return set_err(ctx, FRICO_GPU_EINVAL, "rhs: frequency must be > 0");
    StageTimer tm(ctx, &ctx->stats.rhs_ms);
    ctx->solved = false;
    return rhs_plane_wave(ctx, freq, col, theta, phi, make_double2(Etheta.re, Etheta.im),
                          make_double2(Ephi.re, Ephi.im));
}

extern "C" int frico_gpu_set_rhs(frico_gpu_ctx* ctx, int32_t nrhs, const frico_c128* V, int64_t ldv) {
    FRICO_CTX_CHECK(ctx);
    if (!V || ldv < ctx->n) return set_err(ctx, FRICO_GPU_EINVAL, "set_rhs: bad pointer or ld");
    int rc = frico_gpu_set_nrhs(ctx, nrhs);
    if (rc) return rc;
    rc = cuda_check(ctx, cudaMemcpy2DAsync(ctx->rhs.p, sizeof(double2) * ctx->n, V, sizeof(frico_c128) * ldv,
                                           sizeof(double2) * ctx->n, nrhs, cudaMemcpyHostToDevice, ctx->stream),
                    "upload rhs");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    return rc;
}

extern "C" int frico_gpu_get_rhs(frico_gpu_ctx* ctx, frico_c128* V, int64_t ldv) {
    FRICO_CTX_CHECK(ctx);
    if (ctx->nrhs <= 0) return set_err(ctx, FRICO_GPU_ESTATE, "get_rhs: no right-hand sides");
    if (!V || ldv < ctx->n) return set_err(ctx, FRICO_GPU_EINVAL, "get_rhs: bad pointer or ld");
    int rc = cuda_check(ctx, cudaMemcpy2DAsync(V, sizeof(frico_c128) * ldv, ctx->rhs.p, sizeof(double2) * ctx->n,
                                               sizeof(double2) * ctx->n, ctx->nrhs, cudaMemcpyDeviceToHost, ctx->stream),
                        "download rhs");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    return rc;
}

extern "C" int frico_gpu_solve(frico_gpu_ctx* ctx, frico_c128* I_out, int64_t ldi, int32_t* info) {
    FRICO_CTX_CHECK(ctx);
    if (info) *info = 0;
    if (ctx->nrhs <= 0) return set_err(ctx, FRICO_GPU_ESTATE, "solve: no right-hand sides");
    if (I_out && ldi < ctx->n) return set_err(ctx, FRICO_GPU_EINVAL, "solve: ldi < n");
    const bool mixed = ctx->opt.precision == FRICO_PREC_MIXED;
    const int piv = ctx->opt.pivoting;
    int rc;
    // mixed precision, complex64 factors: without interchanges first (FRICO_PIVOT_AUTO / NONE),
    // partial pivoting when a pivot vanishes or (below) the refinement does not converge
    auto factor_mixed = [&](bool partial) -> int {
        StageTimer tm(ctx, &ctx->stats.factor_ms);
        int r = partial ? lu_factor_fp32(ctx) : lu_factor_nopiv_fp32(ctx);
        ctx->stats.pivoting_used = partial ? FRICO_PIVOT_PARTIAL : FRICO_PIVOT_NONE;
        return r;
    };
    // FP64 LU in place (as zgetrf), Z copied first for the refinement step of the solve
    auto factor_fp64 = [&]() -> int {
        const size_t zb = sizeof(double2) * size_t(ctx->n) * size_t(ctx->n);
        int r = ensure(ctx, ctx->z64_keep, zb);
        if (!r) r = cuda_check(ctx, cudaMemcpyAsync(ctx->z64_keep.p, ctx->z64.p, zb, cudaMemcpyDeviceToDevice, ctx->stream),
                               "keep Z");
        ctx->z64_keep_valid = false;
        if (!r) r = lu_factor_fp64(ctx);
        if (!r) ctx->z64_keep_valid = true;
        return r;
    };
    // factors kept: same precision, or FP64 factors a mixed solve of this Z fell back to
    const bool reuse = ctx->factored && (ctx->factor_prec == ctx->opt.precision ||
                                         (mixed && ctx->factor_prec == FRICO_PREC_FP64));
    if (!reuse) {
        if (!ctx->z_valid) return set_err(ctx, FRICO_GPU_ESTATE, "solve: no impedance matrix (call fill)");
        // a factorisation that stopped part-way left its in-place copy half factored
        if (mixed && ctx->z32_stale && (rc = z64_to_z32(ctx))) return rc;
        ctx->z32_stale = false;
        if (mixed) {
            rc = factor_mixed(piv == FRICO_PIVOT_PARTIAL);
            if (!rc && ctx->info != 0 && piv == FRICO_PIVOT_AUTO) {
                if ((rc = z64_to_z32(ctx))) return rc;
                rc = factor_mixed(true);
            }
        } else {
            StageTimer tm(ctx, &ctx->stats.factor_ms);
            rc = factor_fp64();
            ctx->stats.pivoting_used = FRICO_PIVOT_PARTIAL;
        }
        if (rc) {
            // the factorisation works in place: Z64 (FP64) or the complex64 copy is no longer Z
            if (mixed) ctx->z32_stale = true;
            else ctx->z_valid = false;
            return rc;
        }
        ctx->factored = true;
        ctx->factor_prec = ctx->opt.precision;
        if (!mixed) ctx->z_valid = false;  // Z64 now holds the LU factors, as zgetrf leaves A
    }
    if (info) *info = ctx->info;
    if (ctx->info != 0) {
        char buf[64];
        snprintf(buf, sizeof buf, "ZGETRF singular matrix (info = %d)", ctx->info);
        return set_err(ctx, FRICO_GPU_ESINGULAR, buf);
    }
    ctx->stats.nrhs = ctx->nrhs;
    ctx->stats.refine_iters = 0;
    ctx->stats.refine_residual = 0.0;
    const int64_t n = ctx->n;
    bool fp64_solve = ctx->factor_prec == FRICO_PREC_FP64;
    if (!fp64_solve) {
        {
            StageTimer tm(ctx, &ctx->stats.refine_ms);
            rc = refine_solve(ctx);
        }
        // with classical refinement only, partial pivoting is the next thing to try; GMRES
        // refinement already covers what pivoting would gain, so AUTO goes to FP64 directly
        if (rc == FRICO_GPU_ENOCONV && piv == FRICO_PIVOT_AUTO && ctx->stats.pivoting_used == FRICO_PIVOT_NONE &&
            ctx->opt.refine_mode == FRICO_REFINE_CLASSIC) {
            int rc2 = z64_to_z32(ctx);
            if (!rc2) rc2 = factor_mixed(true);
            if (rc2) return rc2;
            if (ctx->info != 0) {
                if (info) *info = ctx->info;
                return set_err(ctx, FRICO_GPU_ESINGULAR, "singular matrix (complex64 factorisation)");
            }
            StageTimer tm(ctx, &ctx->stats.refine_ms);
            rc = refine_solve(ctx);
        }
        if (rc == FRICO_GPU_ENOCONV && piv == FRICO_PIVOT_AUTO) {
            // complex64 factors cannot refine this system: FP64 LU of Z, assembled again in
            // FP64 arithmetic if the resident one came from the double-float kernels
            if (ctx->z_df) {
                StageTimer tf(ctx, &ctx->stats.fill_ms);
                if ((rc = fill_matrix(ctx, ctx->freq, true))) return rc;
            }
            StageTimer tm(ctx, &ctx->stats.factor_ms);
            rc = factor_fp64();
            if (rc) return rc;
            ctx->factor_prec = FRICO_PREC_FP64;
            ctx->z_valid = false;
            ctx->stats.pivoting_used = FRICO_PIVOT_PARTIAL;
            if (ctx->info != 0) {
                if (info) *info = ctx->info;
                char buf[64];
                snprintf(buf, sizeof buf, "ZGETRF singular matrix (info = %d)", ctx->info);
                return set_err(ctx, FRICO_GPU_ESINGULAR, buf);
            }
            fp64_solve = true;
        }
        ctx->stats.solve_ms = 0.0;
    }
    ctx->stats.precision_used = fp64_solve ? FRICO_PREC_FP64 : FRICO_PREC_MIXED;
    if (fp64_solve) {
        if (!mixed) ctx->stats.refine_ms = 0.0;
        StageTimer tm(ctx, &ctx->stats.solve_ms);
        rc = ensure(ctx, ctx->sol, sizeof(double2) * n * ctx->nrhs);
        if (!rc)
            rc = cuda_check(ctx, cudaMemcpyAsync(ctx->sol.p, ctx->rhs.p, sizeof(double2) * n * ctx->nrhs,
                                                 cudaMemcpyDeviceToDevice, ctx->stream), "copy rhs");
        if (!rc) rc = lu_solve_fp64(ctx, (double2*)ctx->sol.p, ctx->nrhs, n);
        if (!rc && ctx->z64_keep_valid)
            rc = refine_fp64_once(ctx, (const double2*)ctx->z64_keep.p, (const double2*)ctx->rhs.p,
                                  (double2*)ctx->sol.p);
    }
    if (rc && rc != FRICO_GPU_ENOCONV) return rc;
    ctx->solved = true;
    ctx->lumped_col = -1;
    if (I_out) {
        int rc2 = cuda_check(ctx, cudaMemcpy2DAsync(I_out, sizeof(frico_c128) * ldi, ctx->sol.p, sizeof(double2) * n,
                                                    sizeof(double2) * n, ctx->nrhs, cudaMemcpyDeviceToHost, ctx->stream),
                             "download I");
        if (!rc2) rc2 = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
        if (rc2) return rc2;
    }
    return rc;
}

extern "C" int frico_gpu_get_factors(frico_gpu_ctx* ctx, frico_c128* LU, int64_t ld, int32_t* ipiv) {
    FRICO_CTX_CHECK(ctx);
    if (!ctx->factored) return set_err(ctx, FRICO_GPU_ESTATE, "get_factors: not factored");
    const int64_t n = ctx->n;
    int rc = FRICO_GPU_OK;
    if (LU) {
        if (ld < n) return set_err(ctx, FRICO_GPU_EINVAL, "get_factors: ld < n");
        if (ctx->factor_prec == FRICO_PREC_FP64) {
            rc = cuda_check(ctx, cudaMemcpy2DAsync(LU, sizeof(frico_c128) * ld, ctx->z64.p, sizeof(double2) * n,
                                                   sizeof(double2) * n, n, cudaMemcpyDeviceToHost, ctx->stream), "LU");
        } else {
            std::vector<float2> tmp(n * n);
            rc = cuda_check(ctx, cudaMemcpyAsync(tmp.data(), ctx->z32.p, sizeof(float2) * n * n, cudaMemcpyDeviceToHost,
                                                 ctx->stream), "LU32");
            if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
            if (!rc)
                for (int64_t c = 0; c < n; c++)
                    for (int64_t r = 0; r < n; r++) LU[c * ld + r] = {tmp[c * n + r].x, tmp[c * n + r].y};
        }
    }
    if (!rc && ipiv)
        rc = cuda_check(ctx, cudaMemcpyAsync(ipiv, ctx->ipiv.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream),
                        "ipiv");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    return rc;
}

extern "C" int frico_gpu_lump_currents(frico_gpu_ctx* ctx, int32_t col, frico_c128* tri_AJ, frico_c128* tri_AdivJ,
                                       frico_c128* tri_J) {
    FRICO_CTX_CHECK(ctx);
    int rc = check_col(ctx, col);
    if (rc) return rc;
    if (!ctx->solved) return set_err(ctx, FRICO_GPU_ESTATE, "lump_currents: not solved");
    {
        StageTimer tm(ctx, &ctx->stats.lump_ms);
        rc = lump_currents(ctx, col);
    }
    if (rc) return rc;
    const int64_t nt = ctx->nt;
    if (tri_AJ)
        rc = cuda_check(ctx, cudaMemcpyAsync(tri_AJ, ctx->tri_aj.p, sizeof(double2) * 3 * nt, cudaMemcpyDeviceToHost,
                                             ctx->stream), "AJ");
    if (!rc && tri_AdivJ)
        rc = cuda_check(ctx, cudaMemcpyAsync(tri_AdivJ, ctx->tri_adivj.p, sizeof(double2) * nt, cudaMemcpyDeviceToHost,
                                             ctx->stream), "AdivJ");
    if (!rc && tri_J)
        rc = cuda_check(ctx, cudaMemcpyAsync(tri_J, ctx->tri_j.p, sizeof(double2) * 3 * nt, cudaMemcpyDeviceToHost,
                                             ctx->stream), "J");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    return rc;
}

extern "C" int frico_gpu_eval_fields(frico_gpu_ctx* ctx, int32_t col, int64_t npts, const double* P, frico_c128* E,
                                     frico_c128* H) {
    FRICO_CTX_CHECK(ctx);
    int rc = check_col(ctx, col);
    if (rc) return rc;
    if (!ctx->solved) return set_err(ctx, FRICO_GPU_ESTATE, "eval_fields: not solved");
    if (npts <= 0 || !P) return set_err(ctx, FRICO_GPU_EINVAL, "eval_fields: no points");
    StageTimer tm(ctx, &ctx->stats.fields_ms);
    return eval_fields_dev(ctx, col, npts, P, (double2*)E, (double2*)H);
}

// Device-pointer, allocation-free form of frico_gpu_eval_fields (no FRICO
// counterpart). Every pointer is checked to be device memory of the context's
// device before anything is launched, so a host pointer comes back as EINVAL.
static int check_device_ptr(frico_gpu_ctx* ctx, const void* p, const char* what, uintptr_t align) {
    if (!p) return FRICO_GPU_OK;
    if (uintptr_t(p) % align != 0)
        return set_err(ctx, FRICO_GPU_EINVAL, std::string("eval_fields_noalloc: ") + what + " is not " +
                                                  std::to_string(align) + "-byte aligned");
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, FRICO_GPU_EINVAL, std::string("eval_fields_noalloc: ") + what + " is not a device pointer");
    }
    if ((a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) || a.device != ctx->device)
        return set_err(ctx, FRICO_GPU_EINVAL,
                       std::string("eval_fields_noalloc: ") + what + " is not device memory of the context's device");
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_eval_fields_noalloc(frico_gpu_ctx* ctx, int32_t col, int64_t npts, const double* P_dev,
                                             frico_c128* E_dev, frico_c128* H_dev) {
    FRICO_CTX_CHECK(ctx);
    int rc = check_col(ctx, col);
    if (rc) return rc;
    if (!ctx->solved) return set_err(ctx, FRICO_GPU_ESTATE, "eval_fields_noalloc: not solved");
    if (npts <= 0 || !P_dev || (!E_dev && !H_dev))
        return set_err(ctx, FRICO_GPU_EINVAL, "eval_fields_noalloc: need npts > 0, P_dev and E_dev or H_dev");
    if ((rc = check_device_ptr(ctx, P_dev, "P_dev", alignof(double))) ||
        (rc = check_device_ptr(ctx, E_dev, "E_dev", alignof(double2))) ||
        (rc = check_device_ptr(ctx, H_dev, "H_dev", alignof(double2))))
        return rc;
    return eval_fields_noalloc(ctx, col, npts, P_dev, (double2*)E_dev, (double2*)H_dev);
}

extern "C" int frico_gpu_port_values(frico_gpu_ctx* ctx, int32_t col, int32_t n_itf, const int32_t* itf_tags,
                                     frico_c128 V0c, const double* signs, frico_port_values* out) {
    FRICO_CTX_CHECK(ctx);
    int rc = check_col(ctx, col);
    if (rc) return rc;
    if (!ctx->solved) return set_err(ctx, FRICO_GPU_ESTATE, "port_values: not solved");
    if (!out || n_itf < 0 || (n_itf > 0 && !itf_tags)) return set_err(ctx, FRICO_GPU_EINVAL, "port_values: bad args");
    // src/emw_ana_antenna.cpp:76-105
    using cd = std::complex<double>;
    cd V0(V0c.re, V0c.im), current(0.0), power(0.0);
    const int64_t n = ctx->n;
    for (int64_t i = 0; i < n; i++) {
        const frico_rwg& b = ctx->h_rwg[i];
        if (!b.has_interface) continue;
        for (int32_t k = 0; k < n_itf; k++)
            if (b.interface_tag == itf_tags[k]) {
                double2 Ii;
                rc = cuda_check(ctx, cudaMemcpy(&Ii, (const double2*)ctx->sol.p + int64_t(col) * n + i, sizeof(double2),
                                                cudaMemcpyDeviceToHost), "I");
                if (rc) return rc;
                double sign = signs ? signs[i] : 1.0;
                cd I = b.length * cd(Ii.x, Ii.y) * sign;
                current += I;
                power += 0.5 * V0 * std::conj(I);
            }
    }
    cd Z = V0 / current;
    cd gamma = (Z - ctx->opt.Z0) / (Z + ctx->opt.Z0);
    out->voltage = {V0.real(), V0.imag()};
    out->current = {current.real(), current.imag()};
    out->power = {power.real(), power.imag()};
    out->impedance = {Z.real(), Z.imag()};
    out->gamma = {gamma.real(), gamma.imag()};
    out->swr = (1.0 + std::abs(gamma)) / (1.0 - std::abs(gamma));
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_gain(frico_gpu_ctx* ctx, int32_t col, double pwr, double R, int32_t plane, double* G360) {
    FRICO_CTX_CHECK(ctx);
    if (!G360 || plane < 0 || plane > 2) return set_err(ctx, FRICO_GPU_EINVAL, "gain: bad args");
    // src/emw_ana_antenna.cpp:33-65
    std::vector<double> P(3 * 360);
    for (int deg = 0; deg < 360; deg++) {
        double theta = deg * M_PI / 180;
        double c = std::cos(theta), s = std::sin(theta);
        double* p = &P[3 * deg];
        if (plane == FRICO_GAIN_XY) { p[0] = R * c; p[1] = R * s; p[2] = 0.0; }
        else if (plane == FRICO_GAIN_YZ) { p[0] = 0.0; p[1] = R * c; p[2] = R * s; }
        else { p[0] = -R * c; p[1] = 0.0; p[2] = R * s; }
    }
    std::vector<frico_c128> E(3 * 360), H(3 * 360);
    int rc = frico_gpu_eval_fields(ctx, col, 360, P.data(), E.data(), H.data());
    if (rc) return rc;
    using cd = std::complex<double>;
    for (int deg = 0; deg < 360; deg++) {
        const double* p = &P[3 * deg];
        double Rn = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        cd e[3], h[3];
        for (int a = 0; a < 3; a++) {
            e[a] = cd(E[3 * deg + a].re, E[3 * deg + a].im);
            h[a] = std::conj(cd(H[3 * deg + a].re, H[3 * deg + a].im));
        }
        cd S[3] = {0.5 * (e[1] * h[2] - e[2] * h[1]), 0.5 * (e[2] * h[0] - e[0] * h[2]),
                   0.5 * (e[0] * h[1] - e[1] * h[0])};
        double ss = std::norm(S[0]) + std::norm(S[1]) + std::norm(S[2]);
        double Prad = std::sqrt(ss);
        G360[deg] = 4 * M_PI * Rn * Rn * Prad / pwr;
    }
    return FRICO_GPU_OK;
}

static void rcs_from_E(const frico_c128* E, double theta_s, double phi_s, double R, double* vv, double* hh) {
    // bistatic_RCS_unit_Ei, src/emw_ana_bistatic_rcs.cpp:62-82
    using cd = std::complex<double>;
    double th[3] = {std::cos(theta_s) * std::cos(phi_s), std::cos(theta_s) * std::sin(phi_s), -std::sin(theta_s)};
    double ph[3] = {-std::sin(phi_s), std::cos(phi_s), 0.0};
    cd Et(0.0), Ep(0.0);
    for (int a = 0; a < 3; a++) {
        cd e(E[a].re, E[a].im);
        Et += th[a] * e;
        Ep += ph[a] * e;
    }
    *vv = 4.0 * M_PI * R * R * std::norm(Et);
    *hh = 4.0 * M_PI * R * R * std::norm(Ep);
}

static void sph2rect(double R, double theta, double phi, double* p) {
    // src/utils.h:54-61
    p[0] = R * std::cos(phi) * std::sin(theta);
    p[1] = R * std::sin(phi) * std::sin(theta);
    p[2] = R * std::cos(theta);
}

extern "C" int frico_gpu_bistatic_rcs(frico_gpu_ctx* ctx, int32_t col, double R, double* out) {
    FRICO_CTX_CHECK(ctx);
    if (!out) return set_err(ctx, FRICO_GPU_EINVAL, "bistatic_rcs: null output");
    // src/emw_ana_bistatic_rcs.cpp:102-117: theta cut at phi=0, "phi" cut at theta=0
    const double deg2rad = M_PI / 180.0;
    std::vector<double> P(3 * 718);
    for (int i = 0; i < 359; i++) {
        sph2rect(R, deg2rad * i, 0.0, &P[3 * i]);
        sph2rect(R, 0.0, deg2rad * i, &P[3 * (359 + i)]);
    }
    std::vector<frico_c128> E(3 * 718);
    int rc = frico_gpu_eval_fields(ctx, col, 718, P.data(), E.data(), nullptr);
    if (rc) return rc;
    for (int i = 0; i < 359; i++) {
        rcs_from_E(&E[3 * i], deg2rad * i, 0.0, R, &out[4 * i], &out[4 * i + 1]);
        rcs_from_E(&E[3 * (359 + i)], 0.0, deg2rad * i, R, &out[4 * i + 2], &out[4 * i + 3]);
    }
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_rcs_points(frico_gpu_ctx* ctx, int32_t col, double R, int64_t npts, const double* theta,
                                    const double* phi, double* out) {
    FRICO_CTX_CHECK(ctx);
    if (!out || !theta || !phi || npts <= 0) return set_err(ctx, FRICO_GPU_EINVAL, "rcs_points: bad args");
    std::vector<double> P(3 * npts);
    for (int64_t i = 0; i < npts; i++) sph2rect(R, theta[i], phi[i], &P[3 * i]);
    std::vector<frico_c128> E(3 * npts);
    int rc = frico_gpu_eval_fields(ctx, col, npts, P.data(), E.data(), nullptr);
    if (rc) return rc;
    for (int64_t i = 0; i < npts; i++) rcs_from_E(&E[3 * i], theta[i], phi[i], R, &out[2 * i], &out[2 * i + 1]);
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_eval_fields_multi(frico_gpu_ctx* ctx, int32_t col0, int32_t ncols, int64_t npts,
                                           const double* P, frico_c128* E, frico_c128* H) {
    FRICO_CTX_CHECK(ctx);
    if (!ctx->solved) return set_err(ctx, FRICO_GPU_ESTATE, "eval_fields_multi: not solved");
    if (ncols <= 0 || col0 < 0 || col0 + ncols > ctx->nrhs)
        return set_err(ctx, FRICO_GPU_EINVAL, "eval_fields_multi: column range outside [0, nrhs)");
    if (npts <= 0 || !P || (!E && !H)) return set_err(ctx, FRICO_GPU_EINVAL, "eval_fields_multi: bad args");
    StageTimer tm(ctx, &ctx->stats.fields_ms);
    if (!E) {
        std::vector<frico_c128> tmp(size_t(3) * ncols * npts);
        return eval_fields_multi(ctx, col0, ncols, npts, P, (double2*)tmp.data(), (double2*)H);
    }
    return eval_fields_multi(ctx, col0, ncols, npts, P, (double2*)E, (double2*)H);
}

extern "C" int frico_gpu_rcs_points_multi(frico_gpu_ctx* ctx, int32_t col0, int32_t ncols, double R, int64_t npts,
                                          const double* theta, const double* phi, double* out) {
    FRICO_CTX_CHECK(ctx);
    if (!out || !theta || !phi || npts <= 0) return set_err(ctx, FRICO_GPU_EINVAL, "rcs_points_multi: bad args");
    std::vector<double> P(3 * npts);
    for (int64_t i = 0; i < npts; i++) sph2rect(R, theta[i], phi[i], &P[3 * i]);
    std::vector<frico_c128> E(size_t(3) * ncols * npts);
    int rc = frico_gpu_eval_fields_multi(ctx, col0, ncols, npts, P.data(), E.data(), nullptr);
    if (rc) return rc;
    for (int64_t c = 0; c < ncols; c++)
        for (int64_t i = 0; i < npts; i++)
            rcs_from_E(&E[3 * (c * npts + i)], theta[i], phi[i], R, &out[2 * (c * npts + i)],
                       &out[2 * (c * npts + i) + 1]);
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_debug_cgemm(frico_gpu_ctx* ctx, int32_t m, int32_t n, int32_t k, const frico_c64* A,
                                     const frico_c64* B, frico_c64* C, int32_t engine) {
    FRICO_CTX_CHECK(ctx);
    if (m <= 0 || n <= 0 || k <= 0 || !A || !B || !C) return set_err(ctx, FRICO_GPU_EINVAL, "debug_cgemm: bad args");
    if (engine != FRICO_GEMM_SIMT && engine != FRICO_GEMM_TC && engine != FRICO_GEMM_TC_F16)
        return set_err(ctx, FRICO_GPU_EINVAL, "debug_cgemm: engine must be SIMT, TC or TC_F16");
    if (engine != FRICO_GEMM_SIMT && !gemm_tc_available(ctx))
        return set_err(ctx, FRICO_GPU_EINVAL, "tensor-core GEMM engine not available on this device");
    int rc;
    if ((rc = ensure(ctx, ctx->status, sizeof(DeviceStatus)))) return rc;
    if ((rc = cuda_check(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(DeviceStatus), ctx->stream), "status")))
        return rc;
    const size_t sa = size_t(m) * k, sb = size_t(k) * n, sc = size_t(m) * n;
    DevBuf buf;
    if ((rc = ensure(ctx, buf, sizeof(float2) * (sa + sb + sc)))) return rc;
    float2* dA = (float2*)buf.p;
    float2* dB = dA + sa;
    float2* dC = dB + sb;
    rc = cuda_check(ctx, cudaMemcpyAsync(dA, A, sizeof(float2) * sa, cudaMemcpyHostToDevice, ctx->stream), "A");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(dB, B, sizeof(float2) * sb, cudaMemcpyHostToDevice, ctx->stream), "B");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(dC, C, sizeof(float2) * sc, cudaMemcpyHostToDevice, ctx->stream), "C");
    if (!rc)
        rc = engine != FRICO_GEMM_SIMT
                 ? gemm_update_tc(ctx, dC, m, dA, m, dB, k, m, n, k, nullptr, 1, 0, 0, engine == FRICO_GEMM_TC_F16 ? 1 : 0)
                 : gemm_update_simt32(ctx, dC, m, dA, m, dB, k, m, n, k);
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(C, dC, sizeof(float2) * sc, cudaMemcpyDeviceToHost, ctx->stream), "C");
    DeviceStatus hs{};
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(&hs, ctx->status.p, sizeof hs, cudaMemcpyDeviceToHost, ctx->stream), "st");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    release(buf);
    if (!rc && hs.err == FRICO_DEV_ERR_TIMEOUT) rc = set_err(ctx, FRICO_GPU_ETIMEOUT, "tensor-core GEMM wait timed out");
    return rc;
}

extern "C" int frico_gpu_debug_z64(frico_gpu_ctx* ctx, const void** dev_ptr, int64_t* ld) {
    if (!ctx || !dev_ptr || !ld) return FRICO_GPU_EINVAL;
    if (!ctx->z_valid || !ctx->z64.p) return set_err(ctx, FRICO_GPU_ESTATE, "debug_z64: no FP64 Z resident");
    *dev_ptr = ctx->z64.p;
    *ld = ctx->n;
    return FRICO_GPU_OK;
}

extern "C" int frico_gpu_last_stats(frico_gpu_ctx* ctx, frico_gpu_stats* stats) {
    if (!ctx || !stats) return FRICO_GPU_EINVAL;
    *stats = ctx->stats;
    return FRICO_GPU_OK;
}
