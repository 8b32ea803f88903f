// Internal definitions shared by the CUDA translation units of libfrico_gpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>
#include <vector>

#include "frico_gpu.h"

// src/constants.h:24-25
#define FRICO_MU0 1.256637061435917e-06
#define FRICO_EPS0 8.8541878188e-12

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_1_PI
#define M_1_PI 0.31830988618379067154
#endif

namespace frico {

// ---------------------------------------------------------------- complex
template <typename R> struct cvec;
template <> struct cvec<double> { using type = double2; };
template <> struct cvec<float> { using type = float2; };
template <typename R> using cplx = typename cvec<R>::type;

__host__ __device__ __forceinline__ double2 cmake(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ float2 cmake(float r, float i) { return make_float2(r, i); }
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { return {a.x + b.x, a.y + b.y}; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { return {a.x - b.x, a.y - b.y}; }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename C, typename R> __host__ __device__ __forceinline__ C cscale(C a, R s) { return {a.x * s, a.y * s}; }
// acc += a*b as four fused multiply-adds (written as acc += x*y - z*w the compiler forms
// the difference first: a multiply, an FMA and an add per part)
template <typename C> __device__ __forceinline__ void cmac(C& acc, C a, C b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a)*b, four fused multiply-adds
template <typename C> __device__ __forceinline__ void cmac_conj(C& acc, C a, C b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
}
// a - b*c
template <typename C> __host__ __device__ __forceinline__ C cfms(C a, C b, C c) {
    return {a.x - b.x * c.x + b.y * c.y, a.y - b.x * c.y - b.y * c.x};
}
// Complex division a / b as std::complex<double> operator/ computes it in the
// common case (Smith-free textbook form; the inputs here are well scaled).
template <typename C> __host__ __device__ __forceinline__ C cdiv(C a, C b) {
    auto d = b.x * b.x + b.y * b.y;
    return {(a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d};
}
template <typename C> __host__ __device__ __forceinline__ auto cabs1(C a) { return fabs(a.x) + fabs(a.y); }

// ---------------------------------------------------------------- double-float
// FP64 work on the FP32 pipe (many times wider than the FP64 one on this part):
// a value is an unevaluated sum hi + lo of two FP32 numbers (about 47 bits).
// split_df: FP64 d -> h + l by integer operations, |d - h - l| <= 2^-47 |d|;
// zero and subnormal d give 0 + 0, exponents outside [-100, 127] set bad.
__device__ __forceinline__ void split_df(double d, float& h, float& l, int& bad) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned hi = unsigned(u >> 32), lo = unsigned(u);
    const unsigned sg = hi & 0x80000000u;
    const int e = int((hi >> 20) & 0x7FFu);
    const int E = e - 1023;
    const bool zero = e == 0;   // zero or subnormal (below 1e-307): taken as zero
    bad |= (!zero && (E < -100 || E > 127)) ? 1 : 0;
    const int Ec = min(max(E, -100), 127);
    const unsigned mtop = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned b = sg | (unsigned(Ec + 104) << 23);   // 2^(E-23), sign of d
    const float hv = __uint_as_float(sg | (unsigned(Ec + 127) << 23) | mtop);
    const float lv = __fsub_rn(__uint_as_float(b | ((lo & 0x1FFFFFFFu) >> 6)), __uint_as_float(b));
    h = zero ? 0.f : hv;
    l = zero ? 0.f : lv;
}

// (s, t) += a b, a = a1 + a2, b = b1 + b2
__device__ __forceinline__ void df_mac(float& s, float& t, float a1, float a2, float b1, float b2) {
    const float p = __fmul_rn(a1, b1);
    float e = __fmaf_rn(a1, b1, -p);
    e = __fmaf_rn(a1, b2, e);
    e = __fmaf_rn(a2, b1, e);
    const float sn = __fadd_rn(s, p);
    const float v = __fsub_rn(sn, s);
    t = __fadd_rn(t, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(sn, v)), __fsub_rn(p, v)), e));
    s = sn;
}

__device__ __forceinline__ void df_renorm(float& s, float& t) {
    const float sn = __fadd_rn(s, t);
    t = __fsub_rn(t, __fsub_rn(sn, s));
    s = sn;
}

// FP32 value as FP64 by integer operations (normal numbers; subnormals and zero give 0)
__device__ __forceinline__ double f2d_exact(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned e = (u >> 23) & 0xFFu;
    if (e == 0) return 0.0;
    const unsigned long long b = (unsigned long long)(u & 0x80000000u) << 32 |
                                 (unsigned long long)(e - 127u + 1023u) << 52 |
                                 (unsigned long long)(u & 0x7FFFFFu) << 29;
    return __longlong_as_double((long long)b);
}

// ---------------------------------------------------------------- errors
#define FRICO_DEV_ERR_TIMEOUT 1
#define FRICO_DEV_ERR_BOUNDS 2

struct DeviceStatus {
    int err;       // FRICO_DEV_ERR_* (first one wins)
    int info;      // LAPACK-style info of the last factorisation (0 = ok)
    int where;     // diagnostic: which barrier / index gave up
    int df_range;  // the double-float residual met an entry outside its exponent range
};

// ---------------------------------------------------------------- mesh on device
// Per-triangle geometry, 16 doubles: v0, v1, v2, barycentre, area (cross
// product, src/geom_mesh.cpp:71-78), Kahan area (src/quadratures.cpp:41-57), pad.
struct TriGeo {
    double v[9];
    double c[3];
    double area;
    double area_kahan;
    double pad[2];
};

// Device-side RWG table in structure-of-arrays form.
struct RwgDev {
    int32_t* itm;   // T- index
    int32_t* itp;   // T+ index
    double* len;    // edge length
    double* am;     // area T-
    double* ap;     // area T+
    double* vm;     // free vertex of T-  [3n]
    double* vp;     // free vertex of T+  [3n]
    int32_t* itf;   // interface tag or INT32_MIN
};

struct Ctx;

// CUDA graph of the complex64 no-pivot factorisation (see lu_nopiv.cu).
struct LuGraph {
    uintptr_t key[12] = {};
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;
    double gemm_flops = 0.0, gemm_bytes = 0.0;
    size_t prof_used = 0;
};

// Workspace that only grows; freed with the context.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace frico

struct frico_gpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;   // look-ahead stream of the complex64 LU
    cudaEvent_t la_ev[2] = {nullptr, nullptr};
    frico::LuGraph lu_graph;          // captured complex64 factorisation
    frico_gpu_options opt{};
    std::string last_error;

    // mesh
    int64_t nv = 0, nt = 0, n = 0;
    int geo_degree = -1;          // degree the quadrature tables were built for
    int nq = 0;                   // points per triangle at that degree
    frico::DevBuf xyz, tri, trigeo, qp, qps, rwg_itm, rwg_itp, rwg_len, rwg_am, rwg_ap, rwg_vm,
        rwg_vp, rwg_itf;
    frico::DevBuf tri_bf;         // [nt*3] basis index (+1, signed by side) per triangle slot
    // triangles renumbered in order of first use by the RWGs (itm, then itp, in matrix order):
    // the double-float Green table is indexed by these numbers, so the table entries of a tile
    // of RWG pairs lie in a small block of it
    frico::DevBuf tri_new;        // [nt] new number of each triangle
    frico::DevBuf tri_old;        // [nt] triangle of each new number
    void* h_stage = nullptr;      // pinned host staging of the mesh upload (frico_gpu_set_mesh)
    size_t h_stage_bytes = 0;
    std::vector<frico_rwg> h_rwg; // host copy (port values, interfaces)
    std::vector<double> h_xyz;    // host copies of the mesh (sweep lanes are built from them)
    std::vector<int64_t> h_tri;
    int64_t mesh_gen = 0;         // bumped by every set_mesh

    // frequency-sweep lanes: sub-contexts on the same device, one per concurrent frequency
    std::vector<frico_gpu_ctx*> lanes;
    int64_t lanes_mesh_gen = -1;

    // fill
    double freq = 0.0;
    bool z_valid = false;         // Z64 holds the matrix of `freq`
    bool z_df = false;            // ... assembled in double-float (mixed precision only)
    bool z32_stale = false;       // z32 no longer holds Z (a factorisation stopped part-way)
    frico::DevBuf gtab, smom, basis_aux, z64, z32;

    // factorisation / solve
    bool factored = false;
    int factor_prec = -1;         // precision of the resident factors (FP64 after a mixed fallback)
    int32_t info = 0;
    frico::DevBuf z64_keep;          // FP64 drop-in: Z as it was before the in-place factorisation
    bool z64_keep_valid = false;     // z64_keep holds the matrix of the resident FP64 factors
    frico::DevBuf res64;             // FP64 refinement residual
    frico::DevBuf ipiv, perm, panel_ws, status;
    int32_t nrhs = 0;
    frico::DevBuf rhs, sol, rwork, rwork32, dwork32, norms;
    frico::DevBuf dinv, trsv_flags;  // inverted diagonal blocks, chain flags + ticket
    frico::DevBuf tc_ws;             // split operands of the tensor-core trailing update
    frico::DevBuf dinv128;           // no-pivot complex64 LU: 128 x 128 blocks L^-1, U^-1, then the chain M blocks
    frico::DevBuf trsv_x;            // intermediate of the 128-row chained solves
    bool dinv128_valid = false;      // dinv128 belongs to the current complex64 factors
    bool dinv64_stale = false;       // dinv (64-row blocks) not yet computed for them
    int trsv_epoch = 0;
    bool solved = false;

    // post-processing
    frico::DevBuf tri_aj, tri_adivj, tri_j, fld_pts, fld_part, fld_out;

    // adjoint: transposed factors, their inverted diagonal blocks, workspaces
    frico::DevBuf lut, dinv_t, adj_ws, adj_tab;
    frico::DevBuf mlump, mfld;    // multi-column lumped currents and field partial sums
    frico::DevBuf ffws;           // far field as GEMMs: chunk operands, chunk results, FP64 sums
    frico::DevBuf gm_ws;          // GMRES refinement: Arnoldi basis and work vectors
    int32_t lumped_col = -1;

    frico_gpu_stats stats{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> prof_events;   // pairs around profiled launches
    size_t prof_used = 0;
};

namespace frico {

// Returns FRICO_GPU_OK or sets ctx->last_error and returns a code.
int set_err(frico_gpu_ctx* ctx, int code, const std::string& msg);
int cuda_check(frico_gpu_ctx* ctx, cudaError_t e, const char* what);
int ensure(frico_gpu_ctx* ctx, DevBuf& b, size_t bytes);
void release(DevBuf& b);

// Stage timing on the context stream.
struct StageTimer {
    frico_gpu_ctx* ctx;
    double* out;
    StageTimer(frico_gpu_ctx* c, double* o) : ctx(c), out(o) { cudaEventRecord(ctx->ev0, ctx->stream); }
    ~StageTimer() {
        cudaEventRecord(ctx->ev1, ctx->stream);
        if (cudaEventSynchronize(ctx->ev1) == cudaSuccess) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
            *out = ms;
        }
    }
};

// One-time per-device setup (kernel attributes, constant tables): runs `init`
// the first time (device, key) is seen in this process and returns its status;
// a failed init runs again on the next call. Safe to call from several host
// threads (each driving its own context).
enum OnceKey { kOnceDunavant = 0, kOnceGemmTc, kOnceNopivLu, kOnceTrsmLower, kOnceTrsv128, kOnceGemmDf, kOnceGemmPair, kOnceKeys };
int device_once(frico_gpu_ctx* ctx, OnceKey key, int (*init)(frico_gpu_ctx*));

// Limit of the device-side waits on other CTAs (chained solves, grid barrier), in SM cycles.
static const long long kDefaultWaitCycles = 4000000000LL;   // about 2 s at 2 GHz
inline long long wait_limit(const frico_gpu_ctx* ctx) {
    return ctx->opt.wait_limit_cycles > 0 ? (long long)ctx->opt.wait_limit_cycles : kDefaultWaitCycles;
}

// Count one kernel launch on the context (reported as stats.kernel_launches).
inline void count_launch(frico_gpu_ctx* ctx, int64_t k = 1) { ctx->stats.kernel_launches += k; }

// ---- kernels' host launchers (defined in the .cu files) ----
int build_quadrature(frico_gpu_ctx* ctx);                     // fill.cu
int fill_matrix(frico_gpu_ctx* ctx, double freq, bool fp64_only = false);   // fill.cu
int symmetrize(frico_gpu_ctx* ctx);                           // fill.cu
int mirror_upper(frico_gpu_ctx* ctx);                         // fill.cu
int lu_factor_fp64(frico_gpu_ctx* ctx);                       // lu.cu
int lu_factor_fp32(frico_gpu_ctx* ctx);                       // lu.cu
int lu_solve_fp64(frico_gpu_ctx* ctx, double2* B, int nrhs, int64_t ldb);   // lu.cu
int refine_fp64_once(frico_gpu_ctx* ctx, const double2* Zk, const double2* B, double2* X);   // lu.cu
int refine_solve(frico_gpu_ctx* ctx);                         // lu.cu
int trsv_prepare_fp64(frico_gpu_ctx* ctx);                    // trsv.cu
int trsv_prepare_fp32(frico_gpu_ctx* ctx);                    // trsv.cu
int trsv_prepare_nopiv(frico_gpu_ctx* ctx);                   // trsv.cu
int trsv_dinv64_fp32(frico_gpu_ctx* ctx);                     // trsv.cu
int trsv_solve_fp64(frico_gpu_ctx* ctx, double2* W, int nrhs, int64_t ldw);  // trsv.cu
int trsv_solve_fp32(frico_gpu_ctx* ctx, float2* W, int nrhs, int64_t ldw);   // trsv.cu
int trsv_check(frico_gpu_ctx* ctx, DeviceStatus* out = nullptr);   // trsv.cu
int trsv128_prepare(frico_gpu_ctx* ctx, cudaStream_t st);             // trsv.cu
bool gemm_tc_available(frico_gpu_ctx* ctx);                   // gemm_tc.cu
// C (-)= L U on the tensor cores; max_ctas > 0 caps the persistent grid (leaving
// SMs to other streams); reuse_a = 1 keeps the operand split of L from the
// previous call with the same L, m, k; f16 = 1: 3xFP16 operands (else 3xTF32).
int gemm_update_tc(frico_gpu_ctx* ctx, float2* C, int64_t ldc, const float2* L, int64_t ldl,
                   const float2* U, int64_t ldu, int m, int n, int k, cudaEvent_t* ev,
                   int accumulate = 1, int max_ctas = 0, int reuse_a = 0, int f16 = 0);
// Operands of the no-pivot LU's trailing updates written by tc_lu_panel (gemm_tc.cu).
struct TcPanel {
    void* Lah;   // float (3xTF32) or __half (3xFP16, h = 1) operands
    void* Lal;
    void* Ubh;
    void* Ubl;
    int rest, KP;
    int h;
    const float* sc;   // 3xFP16 operand scale s (device)
};
// U11^-1 as the B^ and L11^-1 as the A* operand (hi, lo), written by the
// diagonal-block kernel: TF32 in floats, or (h = 1) FP16, each block scaled by
// the power of two u (l) that puts its largest entry in [2^8, 2^9); the kernel
// then writes 1 / (s u) to *res_l21 and 1 / (l s) to *res_u12 (s = *sc).
struct TcDiagSplit {
    void* uh;
    void* ul;
    void* lh;
    void* ll;
    int h;
    const float* sc;
    float* res_l21;
    float* res_u12;
};
size_t tc_panel_ws_bytes(int64_t n);
int gemm_tc_split_pair(frico_gpu_ctx* ctx, cudaStream_t st, int M, int KP, float* C1, int64_t ldc1, int N1,
                       const float* A1h, const float* A1l, const float* B1h, const float* B1l, float* C2,
                       int64_t ldc2, int N2, const float* A2h, const float* A2l, const float* B2h,
                       const float* B2l);   // gemm_tc.cu
int gemm_tc_dfacc_pair(frico_gpu_ctx* ctx, cudaStream_t st, int M, int KP, int group, int accumulate, float2* C1,
                       int64_t ldc1, int N1, const float* A1h, const float* A1l, const float* B1h, const float* B1l,
                       float2* C2, int64_t ldc2, int N2, const float* A2h, const float* A2l, const float* B2h,
                       const float* B2l);   // gemm_tc.cu
bool fields_gemm_available(frico_gpu_ctx* ctx);                // fields_gemm.cu
int eval_fields_gemm(frico_gpu_ctx* ctx, int ncols, int64_t npts, const double* dP, const double2* AJ,
                     const double2* AD, double2* E_dev, int kc);   // fields_gemm.cu
int tc_diag_split_slots(frico_gpu_ctx* ctx, TcDiagSplit* out);
int tc_lu_scale(frico_gpu_ctx* ctx, const float2* A, int64_t lda, int n);
int tc_lu_panel_split(frico_gpu_ctx* ctx, float2* A, int64_t lda, int k0, int jb, int rest);
int tc_lu_panel(frico_gpu_ctx* ctx, float2* A, int64_t lda, int k0, int jb, int rest, TcPanel* out);
int tc_lu_update(frico_gpu_ctx* ctx, const TcPanel& pn, float2* C, int64_t ldc, int boff, int ncols, int max_ctas,
                 cudaEvent_t* ev);   // gemm_tc.cu
int gemm_update_simt32(frico_gpu_ctx* ctx, float2* C, int64_t ldc, const float2* L, int64_t ldl,
                       const float2* U, int64_t ldu, int m, int n, int k);  // lu.cu
int trsm_lower_unit_f32(frico_gpu_ctx* ctx, float2* A, int64_t lda, int k0, int jb, int cb, int ce);  // lu.cu
cudaEvent_t* prof_event_pair(frico_gpu_ctx* ctx);            // lu.cu
void prof_event_collect(frico_gpu_ctx* ctx);                  // lu.cu
int lu_factor_nopiv_fp32(frico_gpu_ctx* ctx);                 // lu_nopiv.cu
int z64_to_z32(frico_gpu_ctx* ctx);                           // fill.cu
int rhs_delta_gap(frico_gpu_ctx* ctx, double freq, int col, int n_itf, const int32_t* tags,
                  double2 V0, const double* signs);           // fields.cu
int rhs_plane_wave(frico_gpu_ctx* ctx, double freq, int col, double theta, double phi,
                   double2 Eth, double2 Eph);                 // fields.cu
int lump_currents(frico_gpu_ctx* ctx, int col);               // fields.cu
int eval_fields_dev(frico_gpu_ctx* ctx, int col, int64_t npts, const double* P_host,
                    double2* E_host, double2* H_host);        // fields.cu
int eval_fields_noalloc(frico_gpu_ctx* ctx, int col, int64_t npts, const double* P_dev,
                        double2* E_dev, double2* H_dev);      // fields.cu
int64_t eval_fields_noalloc_max_points();                     // fields.cu
void destroy_lanes(frico_gpu_ctx* ctx);                       // sweep.cu
int eval_fields_multi(frico_gpu_ctx* ctx, int col0, int ncols, int64_t npts, const double* P_host,
                      double2* E_host, double2* H_host);     // fields_multi.cu
int trsv_solve_with_fp64(frico_gpu_ctx* ctx, const double2* LU, DevBuf& dinv, double2* W, int nrhs,
                         int64_t ldw);                        // trsv.cu
int trsv_solve_with_fp32(frico_gpu_ctx* ctx, const float2* LU, DevBuf& dinv, float2* W, int nrhs,
                         int64_t ldw);                        // trsv.cu

}  // namespace frico
