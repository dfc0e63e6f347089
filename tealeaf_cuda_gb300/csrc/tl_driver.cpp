// tl_driver.cpp -- the reference's main program restated in C++ above the
// C-ABI: tea_leaf.f90:35-72 -> initialise.f90 / start.f90:25-112 ->
// diffuse.f90:25-101, with the tea.out lines of timestep.f90:58,
// tea_solve.f90:441-462 and field_summary.f90:39-112.
//
// Two ways to run the implicit solve:
//   - default: tl_timestep(), the device-resident solve;
//   - legacy_abi: the host control flow of tea_solve.f90:37-509 calling the
//     reference-named *_kernel_cuda_ entry points one by one, exactly as the
//     reference's Fortran wrappers do.  It is the drop-in path, kept runnable
//     so that tests can show both paths give the same answers.
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tealeaf_capi.h"
#include "tl_host_numerics.h"

namespace {

constexpr double kSmall = 1.0e-16;  // g_small, data.f90:30

// field_summary.f90:96-101, expected final temp of test problems 1..6
const double kQaTemp[7] = {0.0, 157.55084183279294, 106.27221178646569, 99.955877498324000,
                           97.277332050749976, 95.462351583362249, 95.174738768320850};

struct Log {
    FILE *f = nullptr;
    bool echo = false;
    void printf(const char *fmt, ...) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        if (f) fputs(buf, f);
        if (echo) fputs(buf, stdout);
    }
};

// Fortran Ew.d edit descriptor: 0.ddddE+xx right-aligned in w
std::string fortran_e(double x, int w, int d) {
    char body[64];
    if (x == 0.0) {
        std::string z = "0." + std::string(d, '0') + "E+00";
        snprintf(body, sizeof body, "%s", z.c_str());
    } else {
        char tmp[64];
        snprintf(tmp, sizeof tmp, "%.*E", d - 1, std::fabs(x));
        // tmp = "d.ddddE+xx"
        std::string t(tmp);
        size_t epos = t.find('E');
        std::string digits = t.substr(0, 1) + t.substr(2, epos - 2);
        int ex = atoi(t.c_str() + epos + 1) + 1;
        char exs[16];
        if (std::abs(ex) <= 99) snprintf(exs, sizeof exs, "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
        else snprintf(exs, sizeof exs, "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
        snprintf(body, sizeof body, "%s0.%s%s", x < 0 ? "-" : "", digits.c_str(), exs);
    }
    std::string s(body);
    if ((int)s.size() < w) s = std::string(w - s.size(), ' ') + s;
    return s;
}

void print_summary_header(Log &log, double time) {
    log.printf("\n Time %s\n", fortran_e(time, 24, 15).c_str());
    log.printf("%13s%26s%26s%26s%26s%26s\n", "", "Volume", "Mass", "Density", "Energy", "U");
}

void print_summary(Log &log, int step, double vol, double mass, double ie, double temp) {
    log.printf(" step:%7d%s%s%s%s%s\n\n", step, fortran_e(vol, 26, 17).c_str(),
               fortran_e(mass, 26, 17).c_str(), fortran_e(mass / vol, 26, 17).c_str(),
               fortran_e(ie, 26, 17).c_str(), fortran_e(temp, 26, 17).c_str());
}

// ------------------------------------------------------------------------
// tea_solve.f90:37-509 on the host, over the reference-named entry points
// ------------------------------------------------------------------------
struct LegacyState {
    bool first = true;
    double eigmin = 0, eigmax = 0, theta = 0, cn = 0;
};

void halo(const tl_config_t &cf, int field, int depth) {
    if (!cf.reflective_boundary) return;
    int nb[4] = {-1, -1, -1, -1};
    int fl[7] = {0, 0, 0, 0, 0, 0, 0};
    fl[field - 1] = 1;
    update_halo_kernel_cuda_(nb, fl, &depth);
}

void run_ppcg_inner_steps(const tl_config_t &cf, double theta) {
    int inner = cf.ppcg_inner_steps, hd = cf.halo_depth;
    halo(cf, TL_FIELD_U, 1);
    if (inner < 0) return;
    tea_leaf_ppcg_init_sd_new_kernel_cuda_(&theta);
    int nb[4] = {-1, -1, -1, -1};
    for (int cur = 1; cur <= inner; cur += hd) {
        halo(cf, TL_FIELD_SD, hd);
        for (int be = hd - 1; be >= 0; --be) {
            int st = cur + hd - 1 - be;
            tea_leaf_ppcg_inner_kernel_cuda_(&st, &be, nb);
            halo(cf, TL_FIELD_SD, 1);
            if (st == inner) break;
        }
    }
    tea_leaf_ppcg_update_z_kernel_cuda_();
}

int legacy_tea_leaf(const tl_config_t &cf, double dt, LegacyState &S, tl_solve_info_t *info) {
    const auto t0 = std::chrono::steady_clock::now();
    tl_clear_error();
    memset(info, 0, sizeof *info);
    const bool use_cg = cf.solver == TL_SOLVER_CG, use_ch = cf.solver == TL_SOLVER_CHEBYSHEV,
               use_pp = cf.solver == TL_SOLVER_PPCG, use_jac = cf.solver == TL_SOLVER_JACOBI;
    double old_error, error = 0.0, exact_error = 0.0, initial_residual;
    double rro = 0.0, pw, rrn, alpha, beta;
    std::vector<double> cg_alphas(cf.max_iters + 2, 0.0), cg_betas(cf.max_iters + 2, 0.0);
    std::vector<double> ch_alphas, ch_betas;
    int est_itc = 0, cheby_calc_steps = 0, max_cheby_iters = 0, ppcg_inner_iters = 0;
    bool ch_switch_check = false;
    bool fields_p = false, fields_u = false;

    halo(cf, TL_FIELD_DENSITY, cf.halo_depth);
    halo(cf, TL_FIELD_ENERGY1, cf.halo_depth);
    int coef = cf.coefficient;
    int zero[4] = {1, 1, 1, 1};
    int refl = cf.reflective_boundary;
    double rx, ry;
    tea_leaf_common_init_kernel_cuda_(&coef, &dt, &rx, &ry, zero, &refl);
    halo(cf, TL_FIELD_U, 1);
    tea_leaf_calc_residual_cuda_();
    int one = 1, zero_i = 0;
    tea_leaf_calc_2norm_kernel_cuda_(&one, &initial_residual);
    old_error = initial_residual;
    initial_residual = std::sqrt(std::fabs(initial_residual));
    if (use_cg || use_ch || use_pp) {
        tea_leaf_cg_init_kernel_cuda_(&rro);
        halo(cf, TL_FIELD_U, 1);
        halo(cf, TL_FIELD_P, 1);
        fields_p = true;
    } else if (use_jac) {
        fields_u = true;
    }
    int n;
    for (n = 1; n <= cf.max_iters; ++n) {
        if (!ch_switch_check) {
            if (cheby_calc_steps > 0) ch_switch_check = true;
            else if (!S.first && use_pp && n > 1) ch_switch_check = true;
            else if (std::fabs(old_error) <= cf.ch_cg_epslim && n >= cf.ch_cg_presteps) ch_switch_check = true;
        }
        if ((use_ch || use_pp) && ch_switch_check) {
            if (cheby_calc_steps == 0) {
                max_cheby_iters = cf.max_iters - n + 2;
                if (S.first) {
                    double emin, emax;
                    int infoe = tl::tl_calc_eigenvalues(cg_alphas.data() + 1, cg_betas.data() + 1,
                                                        n - 1, &emin, &emax);
                    S.first = false;
                    if (infoe != 0) return TL_ERR_EIGEN;
                    S.eigmin = emin * 0.95;
                    S.eigmax = emax * 1.05;
                }
                int ncoef = use_ch ? max_cheby_iters : cf.ppcg_inner_steps;
                ch_alphas.assign(ncoef > 0 ? ncoef : 1, 0.0);
                ch_betas.assign(ncoef > 0 ? ncoef : 1, 0.0);
                tl::tl_calc_ch_coefs(ch_alphas.data(), ch_betas.data(), S.eigmin, S.eigmax, &S.theta, ncoef);
                if (use_ch) {
                    fields_p = false;
                    fields_u = true;
                } else {
                    tea_leaf_ppcg_init_constants_cuda_(ch_alphas.data(), ch_betas.data(), &ncoef);
                }
                S.cn = S.eigmax / S.eigmin;
                info->switch_n = n;
                if (use_pp) {
                    int st = 2;
                    tea_leaf_ppcg_init_kernel_cuda_(&st, &rro);
                    run_ppcg_inner_steps(cf, S.theta);
                    ppcg_inner_iters += cf.ppcg_inner_steps;
                    st = 3;
                    tea_leaf_ppcg_init_kernel_cuda_(&st, &rro);
                    halo(cf, TL_FIELD_P, 1);
                }
            }
            if (use_ch) {
                if (cheby_calc_steps == 0) {
                    double bb;
                    tea_leaf_calc_2norm_kernel_cuda_(&zero_i, &bb);
                    tea_leaf_cheby_init_kernel_cuda_(ch_alphas.data(), ch_betas.data(), &max_cheby_iters, &S.theta);
                    halo(cf, TL_FIELD_U, 1);
                    int st1 = 1;
                    tea_leaf_cheby_iterate_kernel_cuda_(&st1);
                    tea_leaf_calc_2norm_kernel_cuda_(&one, &old_error);
                    double it_alpha = cf.eps * bb / (4.0 * old_error);
                    double gamm = (std::sqrt(S.cn) - 1.0) / (std::sqrt(S.cn) + 1.0);
                    est_itc = (int)std::lround(std::log(it_alpha) / (2.0 * std::log(gamm)));
                    info->est_itc = est_itc;
                    cheby_calc_steps = 1;
                } else {
                    tea_leaf_cheby_iterate_kernel_cuda_(&cheby_calc_steps);
                    if (n >= est_itc && n % 10 == 0) tea_leaf_calc_2norm_kernel_cuda_(&one, &error);
                }
            } else if (use_pp) {
                tea_leaf_cg_calc_w_kernel_cuda_(&pw);
                tea_leaf_ppcg_store_r_kernel_cuda_();
                tea_leaf_ppcg_calc_2norm_kernel_cuda_(&rro);
                alpha = rro / pw;
                tea_leaf_cg_calc_ur_kernel_cuda_(&alpha, &rrn);
                run_ppcg_inner_steps(cf, S.theta);
                ppcg_inner_iters += cf.ppcg_inner_steps;
                tea_leaf_ppcg_calc_rrn_kernel_cuda_(&rrn);
                beta = rrn / rro;
                tea_leaf_ppcg_calc_p_kernel_cuda_(&beta);
                error = rrn;
                rro = rrn;
            }
            cheby_calc_steps++;
        } else if (use_cg || use_ch || use_pp) {
            fields_p = true;
            tea_leaf_cg_calc_w_kernel_cuda_(&pw);
            alpha = rro / pw;
            cg_alphas[n] = alpha;
            tea_leaf_cg_calc_ur_kernel_cuda_(&alpha, &rrn);
            beta = rrn / rro;
            cg_betas[n] = beta;
            tea_leaf_cg_calc_p_kernel_cuda_(&beta);
            error = rrn;
            rro = rrn;
        } else if (use_jac) {
            tea_leaf_jacobi_solve_kernel_cuda_(&error);
        }
        if (fields_u) halo(cf, TL_FIELD_U, 1);
        if (fields_p) halo(cf, TL_FIELD_P, 1);
        error = std::sqrt(std::fabs(error));
        if (std::fabs(error) < cf.eps * initial_residual) break;
        old_error = error;
    }
    if (cf.check_result) {
        halo(cf, TL_FIELD_U, 1);
        tea_leaf_calc_residual_cuda_();
        tea_leaf_calc_2norm_kernel_cuda_(&one, &exact_error);
        exact_error = std::sqrt(exact_error);
    }
    info->iterations = n - 1;
    info->ppcg_inner_iters = ppcg_inner_iters;
    info->initial_residual = initial_residual;
    info->error = error;
    info->error_ratio = error / initial_residual;
    info->exact_error_ratio = cf.check_result ? exact_error / initial_residual : 0.0;
    info->eigmin = S.eigmin;
    info->eigmax = S.eigmax;
    info->rx = rx;
    info->ry = ry;
    info->status = n > cf.max_iters ? TL_WARN_MAXITER : TL_OK;
    tea_leaf_common_finalise_kernel_cuda_();
    halo(cf, TL_FIELD_ENERGY1, 1);
    info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const char *e = tl_last_error();
    if (e && e[0]) return TL_ERR_CUDA;
    return TL_OK;
}

int legacy_start(const tl_config_t &cf, double *vol, double *mass, double *ie, double *temp) {
    tl_clear_error();
    double dx = (cf.xmax - cf.xmin) / (double)(float)cf.x_cells;
    double dy = (cf.ymax - cf.ymin) / (double)(float)cf.y_cells;
    double xmin = cf.xmin, ymin = cf.ymin;
    initialise_chunk_kernel_cuda_(&xmin, &ymin, &dx, &dy);
    int n = cf.nstates;
    std::vector<double> d(n), e(n), x0(n), x1(n), y0(n), y1(n), rad(n);
    std::vector<int> geo(n);
    for (int s = 0; s < n; ++s) {
        d[s] = cf.states[s].density;
        e[s] = cf.states[s].energy;
        x0[s] = cf.states[s].xmin;
        x1[s] = cf.states[s].xmax;
        y0[s] = cf.states[s].ymin;
        y1[s] = cf.states[s].ymax;
        rad[s] = cf.states[s].radius;
        geo[s] = cf.states[s].geometry;
    }
    int gr = TL_GEOM_RECTANGLE, gc = TL_GEOM_CIRCLE, gp = TL_GEOM_POINT;
    generate_chunk_kernel_cuda_(&n, d.data(), e.data(), x0.data(), x1.data(), y0.data(), y1.data(),
                                rad.data(), geo.data(), &gr, &gc, &gp);
    halo(cf, TL_FIELD_DENSITY, cf.halo_depth);
    halo(cf, TL_FIELD_ENERGY0, cf.halo_depth);
    halo(cf, TL_FIELD_ENERGY1, cf.halo_depth);
    set_field_kernel_cuda_();
    field_summary_kernel_cuda_(vol, mass, ie, temp);
    const char *err = tl_last_error();
    return (err && err[0]) ? TL_ERR_CUDA : TL_OK;
}

// warm start model file: "TLWS0001", int64 count, FP32 parameters
int load_model(tl_chunk_t *ch, const char *path) {
    if (!path) {
        fprintf(stderr, "tea_leaf: tl_warm_start learned needs a model file\n");
        return TL_ERR_ARG;
    }
    FILE *f = fopen(path, "rb");
    if (!f) {
        fprintf(stderr, "tea_leaf: cannot open model %s\n", path);
        return TL_ERR_ARG;
    }
    char magic[8];
    long long n = 0;
    int rc = TL_ERR_ARG;
    if (fread(magic, 1, 8, f) == 8 && memcmp(magic, "TLWS0001", 8) == 0 && fread(&n, 8, 1, f) == 1 &&
        n == tl_warm_start_param_count()) {
        std::vector<float> p((size_t)n);
        if (fread(p.data(), sizeof(float), (size_t)n, f) == (size_t)n)
            rc = tl_set_warm_start_model(ch, p.data(), n);
    } else {
        fprintf(stderr, "tea_leaf: %s is not a warm start model of this build\n", path);
    }
    fclose(f);
    return rc;
}

}  // namespace

extern "C" int tl_run_deck(const char *deck_text, const tl_run_options_t *opt, tl_run_result_t *res) {
    tl_run_options_t o;
    memset(&o, 0, sizeof o);
    if (opt) o = *opt;
    tl_run_result_t r;
    memset(&r, 0, sizeof r);
    tl_config_t cf;
    char err[256];
    int rc = tl_parse_deck(deck_text, &cf, err, sizeof err);
    if (rc) {
        fprintf(stderr, "tea_leaf: deck error: %s\n", err);
        if (res) *res = r;
        return rc;
    }
    Log log;
    log.echo = o.echo != 0;
    if (o.out_path) log.f = fopen(o.out_path, "w");
    log.printf("\n Tea Version    1.000\n GB300 CUDA (sm_103a), %s solve\n\n",
               o.legacy_abi ? "reference entry points" : "device-resident");
    log.printf(" Problem initialised and generated\n");

    tl_chunk_t *ch = nullptr;
    LegacyState S;
    double vol = 0, mass = 0, ie = 0, temp = 0;
    if (o.legacy_abi) {
        rc = tl_default_chunk_init(&cf);
        if (!rc) rc = legacy_start(cf, &vol, &mass, &ie, &temp);
        ch = tl_default_chunk();
    } else {
        rc = tl_chunk_create(&cf, &ch);
        if (!rc) rc = tl_start(ch, &vol, &mass, &ie, &temp);
        if (!rc && cf.warm_start == TL_WARM_LEARNED) rc = load_model(ch, o.model_path);
    }
    if (rc) {
        fprintf(stderr, "tea_leaf: start failed: %s\n", tl_last_error());
        if (log.f) fclose(log.f);
        if (ch && !o.legacy_abi) tl_chunk_destroy(ch);
        if (res) *res = r;
        return rc;
    }
    print_summary_header(log, 0.0);
    print_summary(log, 0, vol, mass, ie, temp);
    if (o.records && o.max_records > 0) {
        tl_step_record_t &rec = o.records[0];
        memset(&rec, 0, sizeof rec);
        rec.has_summary = 1;
        rec.vol = vol;
        rec.mass = mass;
        rec.ie = ie;
        rec.temp = temp;
        r.n_records = 1;
    }
    log.printf(" Starting the calculation\n");

    // diffuse.f90:39-101
    double time = 0.0, dt = cf.dtinit;
    int step = 0;
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        step++;
        if (cf.dtinit <= dt) dt = cf.dtinit;  // timestep.f90 + calc_dt.f90
        log.printf(" Step %7d time %11.7f timestep  %9.2E\n", step, time, dt);
        tl_solve_info_t info;
        if (o.legacy_abi) {
            rc = legacy_tea_leaf(cf, dt, S, &info);
        } else {
            tl_set_dt(ch, dt);
            rc = tl_timestep(ch, &info);
        }
        if (rc < 0) {
            fprintf(stderr, "tea_leaf: solve failed at step %d: %s\n", step, tl_last_error());
            break;
        }
        r.solve_seconds += info.seconds;
        r.total_iterations += info.iterations;
        log.printf("Conduction error %s\n", fortran_e(info.error_ratio, 14, 7).c_str());
        if (cf.check_result) log.printf("EXACT error calculated as%s\n", fortran_e(info.exact_error_ratio, 14, 7).c_str());
        log.printf("Iteration count %8d\n", info.iterations);
        if (cf.solver == TL_SOLVER_PPCG)
            log.printf("PPCG Iteration count%8d (Total %8d)\n", info.ppcg_inner_iters,
                       info.ppcg_inner_iters + info.iterations);
        time += dt;
        bool summ = false;
        if (cf.summary_frequency != 0 && step % cf.summary_frequency == 0) {
            summ = true;
            if (o.legacy_abi) field_summary_kernel_cuda_(&vol, &mass, &ie, &temp);
            else tl_field_summary(ch, &vol, &mass, &ie, &temp);
            print_summary_header(log, time);
            print_summary(log, step, vol, mass, ie, temp);
        }
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        log.printf(" Wall clock %24.15E\n", wall);
        const bool complete = time + kSmall > cf.end_time || step >= cf.end_step ||
                              (o.max_steps > 0 && step >= o.max_steps);
        if (complete) {
            summ = true;
            if (o.legacy_abi) field_summary_kernel_cuda_(&vol, &mass, &ie, &temp);
            else tl_field_summary(ch, &vol, &mass, &ie, &temp);
            print_summary_header(log, time);
            print_summary(log, step, vol, mass, ie, temp);
            if (cf.test_problem >= 1 && cf.test_problem <= 6) {
                r.qa_checked = 1;
                r.qa_diff = std::fabs(100.0 * (temp / kQaTemp[cf.test_problem]) - 100.0);
                r.qa_passed = r.qa_diff < 0.001;
                log.printf("Test problem %4d is within %s%% of the expected solution\n",
                           cf.test_problem, fortran_e(r.qa_diff, 16, 7).c_str());
                log.printf(r.qa_passed ? " This test is considered PASSED\n"
                                       : " This test is considered NOT PASSED\n");
            }
        }
        if (o.records && r.n_records < o.max_records) {
            tl_step_record_t &rec = o.records[r.n_records++];
            memset(&rec, 0, sizeof rec);
            rec.step = step;
            rec.time = time - dt;
            rec.dt = dt;
            rec.solve = info;
            rec.has_summary = summ;
            rec.vol = vol;
            rec.mass = mass;
            rec.ie = ie;
            rec.temp = temp;
            rec.wall = wall;
        }
        if (complete) {
            log.printf("\n Calculation complete\n Tea is finishing\n Wall clock %24.15E\n", wall);
            r.wall_seconds = wall;
            break;
        }
    }
    r.status = rc < 0 ? rc : TL_OK;
    r.steps = step;
    r.vol = vol;
    r.mass = mass;
    r.ie = ie;
    r.temp = temp;
    r.kernel_launches = tl_kernel_launches(ch);
    if (log.f) fclose(log.f);
    if (!o.legacy_abi) tl_chunk_destroy(ch);
    if (res) *res = r;
    return r.status;
}
