// Batched frequency sweep: FRICO's do_sweep loop (src/emw_ana_antenna.cpp:236-282,
// src/emw_ana_bistatic_rcs.cpp:121-160) over the frequencies init_sweep lists
// (src/emw_solver.cpp:460-468).
//
// The frequencies of a sweep are independent systems. A small system does not
// fill the GPU (N = 500..3000: the LU's diagonal-block and triangular-solve
// chains use a handful of SMs), so the sweep runs several frequencies at once:
// each lane is a sub-context with its own stream and buffers, driven by its
// own host thread through the same entry points a single-frequency caller
// uses. Lanes take frequencies from a shared counter. Results per frequency
// do not depend on the lane or the lane count.
//
// Lane count: given by the caller, or chosen by timing. With lanes = 0 and a
// long sweep, the first frequencies warm every candidate lane (allocating its
// buffers), then groups of 1, 2, 4, ... concurrent frequencies are timed on
// warm lanes and the best rate is kept for the rest. All of these frequencies
// are real work whose results are kept.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace frico {

void destroy_lanes(frico_gpu_ctx* ctx) {
    for (frico_gpu_ctx* l : ctx->lanes) frico_gpu_ctx_destroy(l);
    ctx->lanes.clear();
    ctx->lanes_mesh_gen = -1;
}

static int ensure_lanes(frico_gpu_ctx* ctx, int want) {
    if (ctx->lanes_mesh_gen != ctx->mesh_gen) destroy_lanes(ctx);
    while (int(ctx->lanes.size()) < want) {
        frico_gpu_ctx* l = nullptr;
        int rc = frico_gpu_ctx_create(&l, ctx->device, &ctx->opt);
        if (rc) return set_err(ctx, rc, "sweep: cannot create a lane context");
        rc = frico_gpu_set_mesh(l, ctx->nv, ctx->h_xyz.data(), ctx->nt, ctx->h_tri.data(), ctx->n, ctx->h_rwg.data());
        if (rc) {
            std::string msg = frico_gpu_last_error(l);
            frico_gpu_ctx_destroy(l);
            return set_err(ctx, rc, "sweep: lane mesh upload: " + msg);
        }
        ctx->lanes.push_back(l);
    }
    ctx->lanes_mesh_gen = ctx->mesh_gen;
    for (frico_gpu_ctx* l : ctx->lanes) {
        int rc = frico_gpu_set_options(l, &ctx->opt);
        if (rc) return set_err(ctx, rc, "sweep: lane options");
    }
    return FRICO_GPU_OK;
}

namespace {

struct SweepArgs {
    int nfreq;
    const double* freqs;
    int n_itf;
    const int32_t* itf_tags;
    frico_c128 V0;
    const double* signs;
    int n_pw;
    const double* pw;
    int64_t npts;
    const double* P;
    frico_port_values* port_out;
    frico_c128* I_out;
    frico_c128* E_out;
    int nrhs;
    int64_t n;
};

struct Tally {
    std::mutex mu;
    frico_sweep_report rep{};
    int err = FRICO_GPU_OK;
    std::string msg;
    std::atomic<bool> abort{false};
    // Mixed precision: frequencies are visited from the highest down; once three of
    // them have needed the FP64 factorisation, every frequency at or below the third
    // (more ill-conditioned: the EFIE low-frequency regime) is solved in FP64
    // directly. A single fallback can be an isolated resonance; a run of them is
    // the low-frequency regime, where each mixed attempt costs more than FP64.
    static constexpr int kFallbacksForDirect = 3;
    double fp64_at_or_below = -1.0;
    std::vector<double> fallback_freqs;
    std::vector<int> order;   // visiting order -> frequency index
};

// One frequency on one lane, as a single-frequency caller would run it.
int run_frequency(frico_gpu_ctx* lane, const SweepArgs& a, int fi, Tally& t, const frico_gpu_options& opt) {
    const double f = a.freqs[fi];
    const int64_t launches0 = lane->stats.kernel_launches;
    bool direct64 = false;
    if (opt.precision == FRICO_PREC_MIXED) {
        std::lock_guard<std::mutex> lock(t.mu);
        direct64 = f <= t.fp64_at_or_below;
    }
    frico_gpu_options o = opt;
    if (direct64) o.precision = FRICO_PREC_FP64;
    if (lane->opt.precision != o.precision) {
        if (int r = frico_gpu_set_options(lane, &o)) return r;
    }
    int rc = frico_gpu_fill(lane, f, nullptr, 0);
    if (!rc) rc = frico_gpu_set_nrhs(lane, a.nrhs);   // zeroes V (the delta gap accumulates into it)
    double rhs_ms = 0.0;
    int col = 0;
    if (!rc && a.n_itf > 0) {
        rc = frico_gpu_rhs_delta_gap(lane, f, col++, a.n_itf, a.itf_tags, a.V0, a.signs);
        rhs_ms += lane->stats.rhs_ms;
    }
    for (int p = 0; !rc && p < a.n_pw; p++) {
        const double* w = a.pw + 6 * p;
        rc = frico_gpu_rhs_plane_wave(lane, f, col++, w[0], w[1], frico_c128{w[2], w[3]}, frico_c128{w[4], w[5]});
        rhs_ms += lane->stats.rhs_ms;
    }
    int32_t info = 0;
    bool noconv = false;
    if (!rc) {
        frico_c128* I = a.I_out ? a.I_out + int64_t(fi) * a.nrhs * a.n : nullptr;
        rc = frico_gpu_solve(lane, I, a.n, &info);
        if (rc == FRICO_GPU_ENOCONV) {
            noconv = true;
            rc = FRICO_GPU_OK;
        }
    }
    if (!rc && a.port_out && a.n_itf > 0)
        rc = frico_gpu_port_values(lane, 0, a.n_itf, a.itf_tags, a.V0, a.signs, a.port_out + fi);
    double fields_ms = 0.0;   // includes the current lumping of each column
    if (!rc && a.E_out && a.npts > 0) {   // all columns in one pass over (point, triangle) pairs
        rc = frico_gpu_eval_fields_multi(lane, 0, a.nrhs, a.npts, a.P, a.E_out + int64_t(fi) * a.nrhs * a.npts * 3,
                                         nullptr);
        fields_ms += lane->stats.fields_ms;
    }
    std::lock_guard<std::mutex> lock(t.mu);
    if (rc) {
        if (t.err == FRICO_GPU_OK) {
            t.err = rc;
            t.msg = "sweep: frequency " + std::to_string(fi) + " (" + std::to_string(f) +
                    " Hz): " + frico_gpu_last_error(lane);
        }
        t.abort = true;
        return rc;
    }
    const frico_gpu_stats& s = lane->stats;
    frico_sweep_report& r = t.rep;
    r.fill_ms += s.fill_ms;
    r.rhs_ms += rhs_ms;
    r.factor_ms += s.factor_ms;
    r.solve_ms += s.solve_ms;
    r.refine_ms += s.refine_ms;
    r.fields_ms += fields_ms;
    r.max_refine_iters = std::max(r.max_refine_iters, s.refine_iters);
    r.max_refine_residual = std::max(r.max_refine_residual, s.refine_residual);
    if (direct64) {
        r.fp64_direct++;
    } else if (lane->opt.precision == FRICO_PREC_MIXED) {
        if (s.precision_used == FRICO_PREC_FP64) {
            r.fp64_fallbacks++;
            t.fallback_freqs.push_back(f);
            if (int(t.fallback_freqs.size()) >= Tally::kFallbacksForDirect) {
                std::vector<double> v = t.fallback_freqs;
                std::nth_element(v.begin(), v.begin() + (Tally::kFallbacksForDirect - 1), v.end(),
                                 std::greater<double>());
                t.fp64_at_or_below = v[Tally::kFallbacksForDirect - 1];
            }
        } else if (lane->opt.pivoting != FRICO_PIVOT_PARTIAL && s.pivoting_used == FRICO_PIVOT_PARTIAL) {
            r.partial_pivot_fallbacks++;
        }
    }
    if (noconv) r.not_converged++;
    r.kernel_launches += s.kernel_launches - launches0;
    return FRICO_GPU_OK;
}

// Visiting positions [lo, hi) on lanes[0 .. nl), each lane taking the next one.
void run_range(std::vector<frico_gpu_ctx*>& lanes, int nl, const SweepArgs& a, int lo, int hi, Tally& t,
               const frico_gpu_options& opt) {
    std::atomic<int> next{lo};
    auto worker = [&](frico_gpu_ctx* lane) {
        for (;;) {
            if (t.abort) return;
            const int pos = next.fetch_add(1);
            if (pos >= hi) return;
            if (run_frequency(lane, a, t.order[pos], t, opt)) return;
        }
    };
    const int nthreads = std::min(nl, hi - lo);
    if (nthreads <= 1) {
        worker(lanes[0]);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(nthreads);
    for (int i = 0; i < nthreads; i++) th.emplace_back(worker, lanes[i]);
    for (std::thread& x : th) x.join();
}

int default_lanes(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>(16, (12000 + n / 2) / n))); }

}  // namespace

static const int kTuneMinFreqs = 160;  // shorter sweeps take the lane count from N

int sweep(frico_gpu_ctx* ctx, const SweepArgs& a, int lanes, frico_sweep_report* report) {
    using clock = std::chrono::steady_clock;
    const auto t0 = clock::now();
    Tally t;
    t.order.resize(a.nfreq);
    for (int i = 0; i < a.nfreq; i++) t.order[i] = i;
    std::stable_sort(t.order.begin(), t.order.end(), [&](int x, int y) { return a.freqs[x] > a.freqs[y]; });
    int rc;
    // memory cap: Z64 + Z32 + factors' workspaces, about 26 N^2 bytes per lane
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const double per_lane = 26.0 * double(a.n) * double(a.n) + 64.0 * 1024 * 1024;
    const int mem_cap = int(std::max(1.0, std::min(64.0, 0.6 * double(free_b) / per_lane)));
    bool tune = lanes == 0 && a.nfreq >= kTuneMinFreqs;
    int nl = lanes > 0 ? lanes : default_lanes(a.n);
    int lmax = std::min(32, mem_cap);
    if (tune) nl = lmax;
    nl = std::max(1, std::min(nl, std::min(mem_cap, a.nfreq)));
    if (lanes > 0 && mem_cap < std::min(lanes, a.nfreq))
        return set_err(ctx, FRICO_GPU_ENOMEM, "sweep: not enough device memory for " + std::to_string(lanes) + " lanes");
    if ((rc = ensure_lanes(ctx, tune ? lmax : nl))) return rc;
    int done = 0;
    if (tune) {
        // warm every candidate lane on its first frequency
        run_range(ctx->lanes, lmax, a, 0, lmax, t, ctx->opt);
        done = lmax;
        double best_rate = 0.0;
        int best = 1;
        for (int l = 1; l <= lmax && !t.abort && done + 2 * l <= a.nfreq; l *= 2) {
            // two frequencies per lane per round: one round is at least one full wave of l
            const auto s0 = clock::now();
            run_range(ctx->lanes, l, a, done, done + 2 * l, t, ctx->opt);
            const double sec = std::chrono::duration<double>(clock::now() - s0).count();
            done += 2 * l;
            const double rate = double(2 * l) / std::max(sec, 1e-9);
            if (rate > best_rate) {
                best_rate = rate;
                best = l;
            } else if (rate < 0.9 * best_rate) {
                break;
            }
        }
        nl = best;
        t.rep.autotuned = 1;
    }
    if (!t.abort && done < a.nfreq) run_range(ctx->lanes, nl, a, done, a.nfreq, t, ctx->opt);
    t.rep.lanes = nl;
    t.rep.nrhs = a.nrhs;
    t.rep.wall_ms = std::chrono::duration<double, std::milli>(clock::now() - t0).count();
    if (report) *report = t.rep;
    if (t.err) return set_err(ctx, t.err, t.msg);
    if (t.rep.not_converged)
        return set_err(ctx, FRICO_GPU_ENOCONV,
                       "sweep: refinement missed its tolerance at " + std::to_string(t.rep.not_converged) +
                           " frequencies");
    return FRICO_GPU_OK;
}

}  // namespace frico

extern "C" int frico_gpu_sweep(frico_gpu_ctx* ctx, int32_t nfreq, const double* freqs, int32_t n_itf,
                               const int32_t* itf_tags, frico_c128 V0, const double* signs, int32_t n_pw,
                               const double* pw, int64_t npts, const double* P, int32_t lanes,
                               frico_port_values* port_out, frico_c128* I_out, frico_c128* E_out,
                               frico_sweep_report* report) {
    using namespace frico;
    if (!ctx) return FRICO_GPU_EINVAL;
    if (int rc = cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice")) return rc;
    if (ctx->n <= 0) return set_err(ctx, FRICO_GPU_ESTATE, "sweep: no mesh (call frico_gpu_set_mesh)");
    if (nfreq <= 0 || !freqs) return set_err(ctx, FRICO_GPU_EINVAL, "sweep: no frequencies");
    for (int32_t i = 0; i < nfreq; i++)
        if (!(freqs[i] > 0.0)) return set_err(ctx, FRICO_GPU_EINVAL, "sweep: frequencies must be > 0");
    if (n_itf < 0 || n_pw < 0 || (n_itf > 0 && !itf_tags) || (n_pw > 0 && !pw))
        return set_err(ctx, FRICO_GPU_EINVAL, "sweep: bad excitation arguments");
    if (n_itf + n_pw == 0) return set_err(ctx, FRICO_GPU_EINVAL, "sweep: no right-hand side");
    if (port_out && n_itf == 0) return set_err(ctx, FRICO_GPU_EINVAL, "sweep: port values need a delta gap");
    if (E_out && (npts <= 0 || !P)) return set_err(ctx, FRICO_GPU_EINVAL, "sweep: fields need points");
    if (lanes < 0 || lanes > 64) return set_err(ctx, FRICO_GPU_EINVAL, "sweep: lanes must be in [0, 64]");
    SweepArgs a{nfreq, freqs, n_itf, itf_tags, V0, signs, n_pw, pw, npts, P, port_out, I_out, E_out,
                (n_itf > 0 ? 1 : 0) + n_pw, ctx->n};
    return sweep(ctx, a, lanes, report);
}
