// tl_solve.cu -- the device-resident implicit solve (one call of tea_leaf(),
// tea_solve.f90:37-509) for the plain FP64 path.
//
// The reference returns every dot product to the host (a blocking cudaMemcpy
// after each reduction, host_reductions_kernel_cuda.hpp:32) and computes
// alpha, beta and the exit test in Fortran.  Here those scalars live in
// DevScalars: the last CTA of each reducing kernel applies the same formulas,
// so the iteration runs without the host.  Iterations are captured into a CUDA
// graph (kIters iterations per graph); every kernel of an iteration returns at
// once when `done` is set, so a graph launched past convergence is a chain of
// empty kernels.  The host polls the scalars of graph k while graph k+1 runs.
//
// The host still owns what the reference computes on the host once per solve:
// the Lanczos eigenvalue estimate (tqli), the Chebyshev coefficients and the
// Chebyshev iteration estimate.
#include <math.h>
#include <string.h>

#include <chrono>
#include <vector>

#include "tl_internal.cuh"
#include "tl_host_numerics.h"

namespace tl {

namespace {

constexpr int kItersCg = 8;
constexpr int kItersPpcg = 2;
constexpr int kItersCheby = 8;
constexpr int kItersJacobi = 8;

enum Phase { kPhaseCg, kPhasePpcg, kPhaseCheby, kPhaseJacobi };

int halo(Chunk *c, int field, int depth) {
    if (!c->cfg.reflective_boundary) return TL_OK;
    int fl[7] = {0, 0, 0, 0, 0, 0, 0};
    fl[field - 1] = 1;
    return chunk_update_halo(c, fl, depth);
}

// tea_leaf_ppcg.f90:174-230 on one chunk: inner steps of the polynomial
// preconditioner, then z = utemp
int ppcg_inner_steps(Chunk *c, bool fast) {
    const int inner = c->cfg.ppcg_inner_steps, hd = c->h;
    int rc;
    if (c->cfg.precision == TL_PRECISION_MIXED) return mixed_ppcg_inner(c);
    if ((rc = halo(c, TL_FIELD_U, 1))) return rc;
    if (inner < 0) return TL_OK;
    if ((rc = launch_ppcg_init_sd_new(c, c->theta, fast))) return rc;
    for (int cur = 1; cur <= inner; cur += hd) {
        if ((rc = halo(c, TL_FIELD_SD, hd))) return rc;
        for (int be = hd - 1; be >= 0; --be) {
            const int st = cur + hd - 1 - be;
            if ((rc = launch_ppcg_update_r(c, fast))) return rc;
            if ((rc = launch_ppcg_calc_sd_new(c, st, fast))) return rc;
            if ((rc = halo(c, TL_FIELD_SD, 1))) return rc;
            if (st == inner) break;
        }
    }
    return launch_copy(c, c->z, c->utemp, fast);
}

// one iteration of each phase, launched with fast = true (graph body)
int body_cg(Chunk *c) {
    int rc;
    if ((rc = launch_cg_w(c, kEpiCgW, true))) return rc;
    if ((rc = launch_cg_ur(c, 0.0, kEpiCgUr, true))) return rc;
    if ((rc = launch_cg_p(c, 0.0, kEpiFinish, true))) return rc;
    return halo(c, TL_FIELD_P, 1);
}

int body_ppcg(Chunk *c) {
    int rc;
    const bool mixed = c->cfg.precision == TL_PRECISION_MIXED;
    if ((rc = launch_ppcg_w_store_zr(c, true, mixed))) return rc;
    bool did_rrn = false;
    if (mixed) {
        if ((rc = mixed_ppcg_ur_inner(c, &did_rrn))) return rc;
    } else {
        if ((rc = launch_cg_ur(c, 0.0, kEpiNone, true))) return rc;
        if ((rc = ppcg_inner_steps(c, true))) return rc;
    }
    if (!did_rrn && (rc = launch_ppcg_rrn(c, kEpiPpcgRrn, true))) return rc;
    if (mixed && mixed_fused(c)) rc = launch_ppcg_up(c, kEpiFinishNoSwitch, true);
    else rc = launch_ppcg_p(c, 0.0, kEpiFinishNoSwitch, true);
    if (rc) return rc;
    return halo(c, TL_FIELD_P, 1);
}

int body_cheby(Chunk *c) {
    int rc;
    if ((rc = launch_cheby_calc_p(c, 0, kEpiChebyNorm, true))) return rc;
    if ((rc = launch_cheby_calc_u(c, kEpiChebyFinish, true))) return rc;
    return halo(c, TL_FIELD_U, 1);
}

int body_jacobi(Chunk *c) {
    int rc;
    if ((rc = launch_jacobi(c, kEpiJacobi, true))) return rc;
    return halo(c, TL_FIELD_U, 1);
}

// capture `iters` iterations of `body` into *exec once; *kernels receives
// the number of kernel nodes per graph
int capture(Chunk *c, int (*body)(Chunk *), int iters, cudaGraphExec_t *exec, long long *kernels) {
    if (*exec) return TL_OK;
    cudaGraph_t graph = nullptr;
    TL_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = TL_OK;
    const long long before = c->launches;
    c->capturing = true;
    for (int k = 0; k < iters && rc == TL_OK; ++k) rc = body(c);
    c->capturing = false;
    *kernels = c->launches - before;
    c->launches = before;  // captured, not launched
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return TL_OK;
}

}  // namespace

// the profiling form of run_phase: the same iterations launched one kernel
// at a time, each bracketed by CUDA events
static int run_phase_eager(Chunk *c, int (*body)(Chunk *), int iters, int *done_out) {
    int rc;
    for (;;) {
        for (int k = 0; k < iters; ++k)
            if ((rc = body(c))) return rc;
        if ((rc = prof_flush(c))) return rc;
        if ((rc = chunk_sync_scalars(c))) return rc;
        if (c->sc_host->done != kRunning) break;
    }
    *done_out = c->sc_host->done;
    return TL_OK;
}

// run graphs of one phase until the device sets done; returns the final done
int run_phase(Chunk *c, int (*body)(Chunk *), int iters, int phase, int *done_out) {
    if (c->profiling) return run_phase_eager(c, body, iters, done_out);
    cudaGraphExec_t *exec = &c->graphs[phase];
    int rc = capture(c, body, iters, exec, &c->graph_kernels[phase]);
    if (rc) return rc;
    const long long per_graph = c->graph_kernels[phase];
    int slot = 0;
    TL_CUDA(cudaGraphLaunch(*exec, c->stream));
    c->launches += per_graph;
    TL_CUDA(cudaMemcpyAsync(&c->poll_host[slot], c->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, c->stream));
    TL_CUDA(cudaEventRecord(c->poll_ev[slot], c->stream));
    for (;;) {
        const int next = slot ^ 1;
        TL_CUDA(cudaGraphLaunch(*exec, c->stream));
        c->launches += per_graph;
        TL_CUDA(cudaMemcpyAsync(&c->poll_host[next], c->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, c->stream));
        TL_CUDA(cudaEventRecord(c->poll_ev[next], c->stream));
        TL_CUDA(cudaEventSynchronize(c->poll_ev[slot]));
        if (c->poll_host[slot].done != kRunning) break;
        slot = next;
    }
    rc = chunk_sync_scalars(c);
    if (rc) return rc;
    *done_out = c->sc_host->done;
    return TL_OK;
}

int solve_timestep(Chunk *c, tl_solve_info_t *info) {
    const auto t0 = std::chrono::steady_clock::now();
    memset(info, 0, sizeof *info);
    const tl_config_t &cf = c->cfg;
    const int solver = cf.solver;
    const bool use_ch = solver == TL_SOLVER_CHEBYSHEV, use_pp = solver == TL_SOLVER_PPCG;
    const bool krylov = solver == TL_SOLVER_CG || use_ch || use_pp;
    int rc;

    // tea_solve.f90:93-97
    {
        int fl[7] = {1, 0, 1, 0, 0, 0, 0};
        if ((rc = chunk_update_halo(c, fl, c->h))) return rc;
    }
    // tea_leaf_common_init: calcrxry (tea_leaf_kernel_cuda.cu:18-32) + kernels
    const double rx = c->dt / (c->dx * c->dx), ry = c->dt / (c->dy * c->dy);
    c->rx = rx;
    c->ry = ry;
    const int zero[4] = {1, 1, 1, 1};
    if ((rc = launch_common_init(c, cf.coefficient, rx, ry, zero, cf.reflective_boundary))) return rc;
    if ((rc = halo(c, TL_FIELD_U, 1))) return rc;

    // scalars of this solve
    // warm start: u = u^n + the Galerkin combination of the network's and the
    // previous step's directions; the exit test keeps the plain start's residual
    double warm_r0 = 0.0, warm_rr = 0.0;
    const bool warm = cf.warm_start != 0;
    if (warm && (rc = warm_start_or_fallback(c, info, &warm_r0, &warm_rr))) return rc;

    DevScalars &h = *c->sc_host;
    memset(&h, 0, sizeof h);
    h.eps = cf.eps;
    h.epslim = cf.ch_cg_epslim;
    h.max_iters = cf.max_iters;
    h.solver = solver;
    h.first = c->first ? 1 : 0;
    h.presteps = cf.ch_cg_presteps;
    h.ppcg_inner = cf.ppcg_inner_steps;
    h.n = 1;
    h.theta = c->theta;
    if (warm) {
        h.initial_residual = warm_r0;
        h.old_error = warm_rr;
    }
    if ((rc = chunk_push_scalars(c))) return rc;

    if (!warm && (rc = launch_residual(c, kEpiResid))) return rc;
    if (krylov) {
        if ((rc = launch_cg_init(c, kEpiRro))) return rc;
        int fl[7] = {0, 0, 0, 1, 1, 0, 0};
        if ((rc = chunk_update_halo(c, fl, 1))) return rc;
    }
    // mixed-precision PPCG: FP32 copies of the operator and preconditioner
    if (use_pp && cf.precision == TL_PRECISION_MIXED && (rc = mixed_ppcg_prepare(c))) return rc;
    if ((rc = chunk_sync_scalars(c))) return rc;
    info->initial_residual = h.initial_residual;

    if (cf.max_iters < 1) {
        h.n_exit = 1;
        h.done = kMaxIters;
    }

    Phase phase = krylov ? kPhaseCg : kPhaseJacobi;
    bool switching = false;
    // mixed PPCG: the CG presteps of the first solve (which feed the
    // eigenvalue estimates) run in FP32 with FP64 scalars
    bool fp32_presteps = use_pp && cf.precision == TL_PRECISION_MIXED && c->first && !cf.reflective_boundary &&
                         cf.max_iters >= 1;
    if ((use_ch || use_pp) && cf.max_iters >= 1) {
        // the switch test of tea_solve.f90:157-171 at n = 1
        if (fabs(h.old_error) <= cf.ch_cg_epslim && 1 >= cf.ch_cg_presteps) switching = true;
    }
    int done = (cf.max_iters < 1) ? kMaxIters : kRunning;
    int est_itc = 0;

    while (done == kRunning || done == kSwitch) {
        if (switching) {
            switching = false;
            if ((rc = chunk_sync_scalars(c))) return rc;
            const int n = h.n;
            const int max_cheby_iters = cf.max_iters - n + 2;
            if (c->first) {
                std::vector<double> al(n + 1, 0.0), be(n + 1, 0.0);
                if (n > 1) {
                    // on the chunk's own (non-blocking) stream, then wait for it
                    TL_CUDA(cudaMemcpyAsync(al.data(), c->cg_alphas, sizeof(double) * n,
                                            cudaMemcpyDeviceToHost, c->stream));
                    TL_CUDA(cudaMemcpyAsync(be.data(), c->cg_betas, sizeof(double) * n,
                                            cudaMemcpyDeviceToHost, c->stream));
                    TL_CUDA(cudaStreamSynchronize(c->stream));
                }
                double emin = 0.0, emax = 0.0;
                const int info_e = tl_calc_eigenvalues(al.data() + 1, be.data() + 1, n - 1, &emin, &emax);
                c->first = false;
                if (info_e != 0) {
                    set_error("tea_leaf: Error in calculating eigenvalues");
                    info->status = TL_ERR_EIGEN;
                    return TL_ERR_EIGEN;
                }
                c->eigmin = emin * 0.95;
                c->eigmax = emax * 1.05;
            }
            const int ncoef = use_ch ? max_cheby_iters : cf.ppcg_inner_steps;
            std::vector<double> cha(ncoef > 0 ? ncoef : 1), chb(ncoef > 0 ? ncoef : 1);
            tl_calc_ch_coefs(cha.data(), chb.data(), c->eigmin, c->eigmax, &c->theta, ncoef);
            if ((rc = chunk_upload_coefs(c, cha.data(), chb.data(), ncoef))) return rc;
            c->cn = c->eigmax / c->eigmin;
            info->switch_n = n;
            info->eigmin = c->eigmin;
            info->eigmax = c->eigmax;
            h.first = 0;
            h.theta = c->theta;
            h.done = kRunning;
            if (use_pp) {
                // tea_solve.f90:226-250: re-initialise CG with PPCG applied
                if ((rc = chunk_push_scalars(c))) return rc;
                if ((rc = launch_ppcg_init(c, 2, kEpiNone))) return rc;
                if ((rc = ppcg_inner_steps(c, false))) return rc;
                if ((rc = launch_ppcg_init(c, 3, kEpiRro))) return rc;
                if ((rc = halo(c, TL_FIELD_P, 1))) return rc;
                phase = kPhasePpcg;
            } else {
                // tea_leaf_cheby_first_step (tea_leaf_cheby.f90:176-220); its
                // error argument is the caller's old_error
                if ((rc = chunk_push_scalars(c))) return rc;
                if ((rc = launch_norm(c, c->u0, c->u0, kEpiStore))) return rc;
                if ((rc = chunk_sync_scalars(c))) return rc;
                const double bb = h.sum[0];
                if ((rc = launch_cheby_init(c, c->theta))) return rc;
                if ((rc = launch_cheby_calc_u(c, kEpiNone, false))) return rc;
                if ((rc = halo(c, TL_FIELD_U, 1))) return rc;
                if ((rc = launch_cheby_calc_p(c, 1, kEpiNone, false))) return rc;
                if ((rc = launch_cheby_calc_u(c, kEpiNone, false))) return rc;
                if ((rc = launch_norm(c, c->r, c->r, kEpiStore))) return rc;
                if ((rc = chunk_sync_scalars(c))) return rc;
                const double rr = h.sum[0];
                const double it_alpha = cf.eps * bb / (4.0 * rr);
                const double gamm = (sqrt(c->cn) - 1.0) / (sqrt(c->cn) + 1.0);
                est_itc = (int)lround(log(it_alpha) / (2.0 * log(gamm)));
                info->est_itc = est_itc;
                // end of iteration n (tea_solve.f90:284-417) on the host
                h.cheby_calc_steps = 2;
                h.est_itc = est_itc;
                if ((rc = halo(c, TL_FIELD_U, 1))) return rc;
                const double e = sqrt(fabs(h.error));
                h.error = e;
                if (fabs(e) < cf.eps * h.initial_residual) {
                    h.done = kConverged;
                    h.n_exit = n;
                } else {
                    h.old_error = e;
                    h.n = n + 1;
                    if (h.n > cf.max_iters) {
                        h.done = kMaxIters;
                        h.n_exit = h.n;
                    }
                }
                if ((rc = chunk_push_scalars(c))) return rc;
                done = h.done;
                phase = kPhaseCheby;
                if (done != kRunning) break;
            }
        }
        switch (phase) {
        case kPhaseCg:
            if (fp32_presteps) {
                fp32_presteps = false;
                rc = mixed_ppcg_presteps(c, &done);
                // an FP32 residual below tl_eps is not the FP64 one: let PPCG
                // confirm it (unless there was nothing to solve)
                if (!rc && done == kConverged && h.n > 1) {
                    h.done = kSwitch;
                    if ((rc = chunk_push_scalars(c))) return rc;
                    done = kSwitch;
                }
            } else {
                rc = run_phase(c, body_cg, kItersCg, kPhaseCg, &done);
            }
            break;
        case kPhasePpcg:
            rc = run_phase(c, body_ppcg, kItersPpcg, kPhasePpcg, &done);
            break;
        case kPhaseCheby:
            rc = run_phase(c, body_cheby, kItersCheby, kPhaseCheby, &done);
            break;
        case kPhaseJacobi:
            rc = run_phase(c, body_jacobi, kItersJacobi, kPhaseJacobi, &done);
            break;
        }
        if (rc) return rc;
        if (done == kSwitch) switching = true;
    }
    if ((rc = chunk_sync_scalars(c))) return rc;

    info->iterations = h.n_exit - 1;
    info->error = h.error;
    info->initial_residual = h.initial_residual;
    info->error_ratio = h.error / h.initial_residual;
    if (use_pp && info->switch_n > 0)
        info->ppcg_inner_iters = cf.ppcg_inner_steps * (h.ppcg_iters + 1);
    info->status = done == kConverged ? TL_OK
                   : done == kMaxIters ? TL_WARN_MAXITER
                                       : TL_ERR_BREAKDOWN;
    if (done == kBreakdown) set_error("tea_leaf: breakdown (NaN in the Krylov scalars) at iteration %d", h.n_exit);

    if (cf.check_result) {
        // tea_solve.f90:421-437
        if ((rc = halo(c, TL_FIELD_U, 1))) return rc;
        if ((rc = launch_residual(c, kEpiStore))) return rc;
        if ((rc = chunk_sync_scalars(c))) return rc;
        info->exact_error_ratio = sqrt(h.sum[0]) / info->initial_residual;
    }
    // tea_leaf_finalise + halo of energy1 (tea_solve.f90:467-476)
    if ((rc = launch_finalise(c))) return rc;
    if ((rc = halo(c, TL_FIELD_ENERGY1, 1))) return rc;
    TL_CUDA(cudaStreamSynchronize(c->stream));
    info->eigmin = c->eigmin;
    info->eigmax = c->eigmax;
    info->rx = rx;
    info->ry = ry;
    if ((rc = prof_flush(c))) return rc;
    info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return info->status < 0 ? info->status : TL_OK;
}

}  // namespace tl
