// tl_legacy.cu -- the reference's extern "C" entry points, same names and
// by-reference arguments as UK-MAC/TeaLeaf_CUDA's *_kernel_cuda.cu files, so
// the reference's Fortran wrappers link against this library unchanged.  They
// act on the process-wide default chunk (the reference's `cuda_chunk`,
// init_cuda.cu:33).  Scalar results are returned synchronously, as in the
// reference (a device-to-host copy after every reduction); errors are recorded
// for tl_last_error() instead of aborting the process.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "tl_internal.cuh"

namespace tl {
int default_chunk_replace(const tl_config_t *cfg);
Chunk *default_chunk();
}  // namespace tl

using namespace tl;

namespace {

Chunk *need_chunk(const char *who) {
    Chunk *c = default_chunk();
    if (!c) set_error("%s: initialise_cuda_ has not been called", who);
    return c;
}

double read_sum(Chunk *c, int v) {
    if (chunk_sync_scalars(c) != TL_OK) return NAN;
    return c->sc_host->sum[v];
}

// the C++ scan of tea.in in init_cuda.cu:63-163 / cuda_strings.cu:7-84:
// the first line (without '!') containing the name; its text after '='
std::string match_param(const std::vector<std::string> &lines, const char *name) {
    for (const std::string &l : lines) {
        if (l.find('!') != std::string::npos) continue;
        if (l.find(name) == std::string::npos) continue;
        size_t eq = l.find('=');
        if (eq != std::string::npos) return l.substr(eq + 1);
        return std::string(name);
    }
    return std::string();
}

int read_int(const std::vector<std::string> &lines, const char *name) {
    std::string s = match_param(lines, name);
    if (s.empty()) return -1;
    std::stringstream ss(s);
    int v;
    if (!(ss >> v)) return -1;
    return v;
}

}  // namespace

extern "C" {

// init_cuda.cu:35-167
void initialise_cuda_(int *x_min, int *x_max, int *y_min, int *y_max) {
    tl_config_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.x_cells = *x_max - *x_min + 1;
    cfg.y_cells = *y_max - *y_min + 1;
    cfg.max_iters = 1000;
    cfg.eps = 1e-10;
    cfg.coefficient = TL_COEF_CONDUCTIVITY;
    cfg.ppcg_inner_steps = 64;
    std::vector<std::string> lines;
    std::ifstream in("tea.in");
    if (!in.is_open()) {
        set_error("initialise_cuda_: Input file not found");
        return;
    }
    for (std::string l; std::getline(in, l);) lines.push_back(l);
    cfg.profiler_on = !match_param(lines, "profiler_on").empty();
    cfg.cuda_device = std::max(0, read_int(lines, "cuda_device"));
    cfg.halo_depth = read_int(lines, "halo_depth");
    if (cfg.halo_depth < 1) {
        set_error("initialise_cuda_: Halo exchange depth unspecified or was too small");
        return;
    }
    if (!match_param(lines, "tl_use_ppcg").empty()) cfg.solver = TL_SOLVER_PPCG;
    else if (!match_param(lines, "tl_use_chebyshev").empty()) cfg.solver = TL_SOLVER_CHEBYSHEV;
    else if (!match_param(lines, "tl_use_cg").empty()) cfg.solver = TL_SOLVER_CG;
    else cfg.solver = TL_SOLVER_JACOBI;
    std::string pc = match_param(lines, "tl_preconditioner_type");
    std::transform(pc.begin(), pc.end(), pc.begin(), ::tolower);
    if (pc.find("jac_diag") != std::string::npos) cfg.precond = TL_PREC_JAC_DIAG;
    else if (pc.find("jac_block") != std::string::npos) cfg.precond = TL_PREC_JAC_BLOCK;
    else cfg.precond = TL_PREC_NONE;
    cfg.reflective_boundary = !match_param(lines, "reflective_boundary").empty();
    int mi = read_int(lines, "tl_max_iters");
    if (mi > 0) cfg.max_iters = mi;
    default_chunk_replace(&cfg);
}

// initialise_chunk_kernel_cuda.cu:28-32
void initialise_chunk_kernel_cuda_(double *d_xmin, double *d_ymin, double *d_dx, double *d_dy) {
    Chunk *c = need_chunk("initialise_chunk_kernel_cuda_");
    if (c) chunk_initialise_mesh(c, *d_xmin, *d_ymin, *d_dx, *d_dy);
}

// generate_chunk_kernel_cuda.cu:28-110
void generate_chunk_kernel_cuda_(const int *number_of_states, const double *state_density,
                                 const double *state_energy, const double *state_xmin,
                                 const double *state_xmax, const double *state_ymin,
                                 const double *state_ymax, const double *state_radius,
                                 const int *state_geometry, const int *g_rect, const int *g_circ,
                                 const int *g_point) {
    Chunk *c = need_chunk("generate_chunk_kernel_cuda_");
    if (!c) return;
    const int n = *number_of_states;
    std::vector<tl_state_t> st(n > 0 ? n : 1);
    for (int s = 0; s < n; ++s) {
        st[s].density = state_density[s];
        st[s].energy = state_energy[s];
        st[s].xmin = state_xmin[s];
        st[s].xmax = state_xmax[s];
        st[s].ymin = state_ymin[s];
        st[s].ymax = state_ymax[s];
        st[s].radius = state_radius[s];
        const int gg = state_geometry[s];
        st[s].geometry = gg == *g_rect ? TL_GEOM_RECTANGLE
                         : gg == *g_circ ? TL_GEOM_CIRCLE
                         : gg == *g_point ? TL_GEOM_POINT
                                          : 0;
    }
    tl_state_t *sdev = nullptr;
    if (device_malloc((void **)&sdev, sizeof(tl_state_t) * st.size()) != cudaSuccess) {
        set_error("generate_chunk_kernel_cuda_: cudaMalloc failed");
        return;
    }
    cudaMemcpyAsync(sdev, st.data(), sizeof(tl_state_t) * st.size(), cudaMemcpyHostToDevice, c->stream);
    launch_generate(c, n, sdev);
    cudaStreamSynchronize(c->stream);
    cudaFree(sdev);
}

// set_field_kernel_cuda.cu:4-8
void set_field_kernel_cuda_(void) {
    Chunk *c = need_chunk("set_field_kernel_cuda_");
    if (c) launch_set_field(c);
}

// field_summary_kernel_cuda.cu:30-47
void field_summary_kernel_cuda_(double *vol, double *mass, double *ie, double *temp) {
    Chunk *c = need_chunk("field_summary_kernel_cuda_");
    if (!c) return;
    if (launch_field_summary(c) != TL_OK || chunk_sync_scalars(c) != TL_OK) return;
    *vol = c->sc_host->sum[0];
    *mass = c->sc_host->sum[1];
    *ie = c->sc_host->sum[2];
    *temp = c->sc_host->sum[3];
}

// update_halo_kernel_cuda.cu:31-85: mirror the external faces of the
// selected fields (density, energy0, energy1, u, p, sd, r)
void update_halo_kernel_cuda_(const int *chunk_neighbours, const int *fields, const int *depth) {
    Chunk *c = need_chunk("update_halo_kernel_cuda_");
    if (!c) return;
    for (int f = 0; f < 4; ++f)
        if (chunk_neighbours[f] != -1) {
            set_error("update_halo_kernel_cuda_: only a single chunk (all faces external) is supported");
            return;
        }
    double *arr[7] = {c->density, c->energy0, c->energy1, c->u, c->p, c->sd, c->r};
    for (int k = 0; k < 7; ++k)
        if (fields[k] == 1) launch_reflect(c, arr[k], *depth);
}

// pack_kernel_cuda.cu:7-19: MPI halo buffers; one chunk has no neighbours
void cuda_pack_buffers_(int *, int *, int *, int *, double *) {
    set_error("cuda_pack_buffers_: no MPI neighbours on a single chunk");
}
void cuda_unpack_buffers_(int *, int *, int *, int *, double *) {
    set_error("cuda_unpack_buffers_: no MPI neighbours on a single chunk");
}

// tea_leaf_kernel_cuda.cu:233-283 (calcrxry reads celldx/celldy at the halo
// edge; rx and ry are returned)
void tea_leaf_common_init_kernel_cuda_(const int *coefficient, double *dt, double *rx, double *ry,
                                       int *zero_boundary, int *reflective_boundary) {
    Chunk *c = need_chunk("tea_leaf_common_init_kernel_cuda_");
    if (!c) return;
    if (*coefficient != TL_COEF_CONDUCTIVITY && *coefficient != TL_COEF_RECIP_CONDUCTIVITY) {
        set_error("tea_leaf_common_init_kernel_cuda_: Unknown coefficient %d", *coefficient);
        return;
    }
    *rx = *dt / (c->dx * c->dx);
    *ry = *dt / (c->dy * c->dy);
    c->rx = *rx;
    c->ry = *ry;
    launch_common_init(c, *coefficient, *rx, *ry, zero_boundary, *reflective_boundary);
}

void tea_leaf_common_finalise_kernel_cuda_(void) {
    Chunk *c = need_chunk("tea_leaf_common_finalise_kernel_cuda_");
    if (c) launch_finalise(c);
}

void tea_leaf_calc_residual_cuda_(void) {
    Chunk *c = need_chunk("tea_leaf_calc_residual_cuda_");
    if (c) launch_residual(c, kEpiNone);
}

// tea_leaf_kernel_cuda.cu:56-87
void tea_leaf_calc_2norm_kernel_cuda_(int *norm_array, double *norm) {
    Chunk *c = need_chunk("tea_leaf_calc_2norm_kernel_cuda_");
    if (!c) return;
    int rc;
    if (*norm_array == 0) rc = launch_norm(c, c->u0, c->u0, kEpiStore);
    else if (*norm_array == 1) rc = launch_norm(c, c->r, c->r, kEpiStore);
    else if (*norm_array == 2)
        rc = launch_norm(c, c->r, c->cfg.precond != TL_PREC_NONE ? c->z : c->r, kEpiStore);
    else {
        set_error("Invalid value '%d' for norm_array passed, should be [0, 1, 2]", *norm_array);
        return;
    }
    if (rc == TL_OK) *norm = read_sum(c, 0);
}

void tea_leaf_cg_init_kernel_cuda_(double *rro) {
    Chunk *c = need_chunk("tea_leaf_cg_init_kernel_cuda_");
    if (c && launch_cg_init(c, kEpiStore) == TL_OK) *rro = read_sum(c, 0);
}

void tea_leaf_cg_calc_w_kernel_cuda_(double *pw) {
    Chunk *c = need_chunk("tea_leaf_cg_calc_w_kernel_cuda_");
    if (c && launch_cg_w(c, kEpiStore, false) == TL_OK) *pw = read_sum(c, 0);
}

void tea_leaf_cg_calc_ur_kernel_cuda_(double *alpha, double *rrn) {
    Chunk *c = need_chunk("tea_leaf_cg_calc_ur_kernel_cuda_");
    if (c && launch_cg_ur(c, *alpha, kEpiStore, false) == TL_OK) *rrn = read_sum(c, 0);
}

void tea_leaf_cg_calc_p_kernel_cuda_(double *beta) {
    Chunk *c = need_chunk("tea_leaf_cg_calc_p_kernel_cuda_");
    if (c) launch_cg_p(c, *beta, kEpiNone, false);
}

// tea_leaf_kernel_cuda.cu:106-122: upload, init_p, calc_u
void tea_leaf_cheby_init_kernel_cuda_(const double *ch_alphas, const double *ch_betas, int *n_coefs,
                                      const double *theta) {
    Chunk *c = need_chunk("tea_leaf_cheby_init_kernel_cuda_");
    if (!c) return;
    if (chunk_upload_coefs(c, ch_alphas, ch_betas, *n_coefs) != TL_OK) return;
    if (launch_cheby_init(c, *theta) != TL_OK) return;
    launch_cheby_calc_u(c, kEpiNone, false);
}

// tea_leaf_kernel_cuda.cu:124-135
void tea_leaf_cheby_iterate_kernel_cuda_(const int *cheby_calc_step) {
    Chunk *c = need_chunk("tea_leaf_cheby_iterate_kernel_cuda_");
    if (!c) return;
    if (launch_cheby_calc_p(c, *cheby_calc_step, kEpiNone, false) != TL_OK) return;
    launch_cheby_calc_u(c, kEpiNone, false);
}

void tea_leaf_ppcg_init_constants_cuda_(const double *ch_alphas, const double *ch_betas,
                                        int *n_inner_steps) {
    Chunk *c = need_chunk("tea_leaf_ppcg_init_constants_cuda_");
    if (c) chunk_upload_coefs(c, ch_alphas, ch_betas, *n_inner_steps);
}

void tea_leaf_ppcg_init_kernel_cuda_(const int *step, double *rro) {
    Chunk *c = need_chunk("tea_leaf_ppcg_init_kernel_cuda_");
    if (c && launch_ppcg_init(c, *step, kEpiStore) == TL_OK) *rro = read_sum(c, 0);
}

void tea_leaf_ppcg_init_sd_kernel_cuda_(const double *theta) {
    Chunk *c = need_chunk("tea_leaf_ppcg_init_sd_kernel_cuda_");
    if (c) launch_ppcg_init_sd(c, *theta);
}

void tea_leaf_ppcg_init_sd_new_kernel_cuda_(const double *theta) {
    Chunk *c = need_chunk("tea_leaf_ppcg_init_sd_new_kernel_cuda_");
    if (c) launch_ppcg_init_sd_new(c, *theta, false);
}

void tea_leaf_ppcg_store_r_kernel_cuda_(void) {
    Chunk *c = need_chunk("tea_leaf_ppcg_store_r_kernel_cuda_");
    if (c) launch_copy(c, c->r_store, c->r, false);
}

void tea_leaf_ppcg_update_z_kernel_cuda_(void) {
    Chunk *c = need_chunk("tea_leaf_ppcg_update_z_kernel_cuda_");
    if (c) launch_copy(c, c->z, c->utemp, false);
}

void tea_leaf_ppcg_calc_rrn_kernel_cuda_(double *norm) {
    Chunk *c = need_chunk("tea_leaf_ppcg_calc_rrn_kernel_cuda_");
    if (c && launch_ppcg_rrn(c, kEpiStore, false) == TL_OK) *norm = read_sum(c, 0);
}

// tea_leaf_kernel_cuda.cu:418-486: with every face external the matrix-power
// range collapses to the interior whatever bounds_extra is
void tea_leaf_ppcg_inner_kernel_cuda_(int *ppcg_cur_step, int *bounds_extra, int *chunk_neighbours) {
    Chunk *c = need_chunk("tea_leaf_ppcg_inner_kernel_cuda_");
    if (!c) return;
    (void)bounds_extra;
    for (int f = 0; f < 4; ++f)
        if (chunk_neighbours[f] != -1) {
            set_error("tea_leaf_ppcg_inner_kernel_cuda_: only a single chunk is supported");
            return;
        }
    if (launch_ppcg_update_r(c, false) != TL_OK) return;
    launch_ppcg_calc_sd_new(c, *ppcg_cur_step, false);
}

void tea_leaf_ppcg_calc_2norm_kernel_cuda_(double *norm) {
    Chunk *c = need_chunk("tea_leaf_ppcg_calc_2norm_kernel_cuda_");
    if (c && launch_ppcg_zr(c, kEpiStore, false) == TL_OK) *norm = read_sum(c, 0);
}

void tea_leaf_ppcg_calc_p_kernel_cuda_(double *beta) {
    Chunk *c = need_chunk("tea_leaf_ppcg_calc_p_kernel_cuda_");
    if (c) launch_ppcg_p(c, *beta, kEpiNone, false);
}

void tea_leaf_jacobi_solve_kernel_cuda_(double *error) {
    Chunk *c = need_chunk("tea_leaf_jacobi_solve_kernel_cuda_");
    if (c && launch_jacobi(c, kEpiStore, false) == TL_OK) *error = read_sum(c, 0);
}

}  // extern "C"
