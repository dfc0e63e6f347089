// tl_chunk.cu -- chunk runtime: device memory, mesh, fields, errors and the
// tl_* handle API.  Replaces the reference's TealeafCudaChunk
// (cuda_common.hpp:202-388, init_cuda.cu:50-413): one stream per chunk,
// 256-byte aligned rows, status codes instead of MPI_Abort.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include "tl_internal.cuh"

namespace tl {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char *what) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TL_ERR_ALLOC : TL_ERR_CUDA;
}

double *field_ptr(Chunk *c, int field) {
    switch (field) {
    case TL_FIELD_DENSITY: return c->density;
    case TL_FIELD_ENERGY0: return c->energy0;
    case TL_FIELD_ENERGY1: return c->energy1;
    case TL_FIELD_U: return c->u;
    case TL_FIELD_P: return c->p;
    case TL_FIELD_SD: return c->sd;
    case TL_FIELD_R: return c->r;
    case TL_FIELD_U0: return c->u0;
    case TL_FIELD_W: return c->w;
    case TL_FIELD_Z: return c->z;
    case TL_FIELD_KX: return c->kx;
    case TL_FIELD_KY: return c->ky;
    case TL_FIELD_MI: return c->mi;
    case TL_FIELD_CP: return c->cp;
    case TL_FIELD_BFP: return c->bfp;
    case TL_FIELD_VOLUME: return c->volume;
    case TL_FIELD_RTEMP: return c->rtemp;
    case TL_FIELD_UTEMP: return c->utemp;
    case TL_FIELD_R_STORE: return c->r_store;
    default: return nullptr;
    }
}

// Failure injection for tests of the allocation-failure paths (set by
// tl_test_fail_alloc): when the countdown reaches zero, one device
// allocation reports cudaErrorMemoryAllocation without calling cudaMalloc.
static std::atomic<int> g_fail_alloc_countdown{0};

cudaError_t device_malloc(void **p, size_t bytes) {
    int n = g_fail_alloc_countdown.load();
    while (n > 0 && !g_fail_alloc_countdown.compare_exchange_weak(n, n - 1)) {
    }
    if (n == 1) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

static int dalloc(Chunk *c, void **p, size_t bytes) {
    cudaError_t e = device_malloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    c->allocations.push_back(*p);
    e = cudaMemsetAsync(*p, 0, bytes, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    return TL_OK;
}

static void chunk_release(Chunk *c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    mixed_free(c);
    warm_free(c);
    for (cudaGraphExec_t g : c->graphs)
        if (g) cudaGraphExecDestroy(g);
    for (void *p : c->allocations) cudaFree(p);
    for (auto &p : c->ev_pending) c->ev_pool.push_back(p.second);
    for (auto &p : c->ev_pool) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    if (c->sc_host) cudaFreeHost(c->sc_host);
    for (int k = 0; k < 2; ++k)
        if (c->poll_ev[k]) cudaEventDestroy(c->poll_ev[k]);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

static int chunk_alloc(const tl_config_t *cfg, Chunk **out) {
    *out = nullptr;
    if (cfg->x_cells < 1 || cfg->y_cells < 1 || cfg->halo_depth < 1 || cfg->max_iters < 0) {
        set_error("invalid grid: x_cells=%d y_cells=%d halo_depth=%d", cfg->x_cells, cfg->y_cells,
                  cfg->halo_depth);
        return TL_ERR_ARG;
    }
    if ((long long)(cfg->x_cells + 2 * cfg->halo_depth) * (cfg->y_cells + 2 * cfg->halo_depth) >
        (1LL << 40)) {
        set_error("grid too large");
        return TL_ERR_ARG;
    }
    cudaError_t e = cudaSetDevice(cfg->cuda_device < 0 ? 0 : cfg->cuda_device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    Chunk *c = new Chunk();  // value-initialised: every scalar member starts at zero
    c->cfg = *cfg;
    c->device = cfg->cuda_device < 0 ? 0 : cfg->cuda_device;
    c->nx = cfg->x_cells;
    c->ny = cfg->y_cells;
    c->h = cfg->halo_depth;
    c->lead = (32 - c->h % 32) % 32;
    c->pitch = ((c->nx + 2 * c->h + 31) / 32) * 32;
    c->rows = c->ny + 2 * c->h;
    c->alloc_elems = (size_t)c->lead + (size_t)c->pitch * (size_t)c->rows + 32;
    c->g.nx = c->nx;
    c->g.ny = c->ny;
    c->g.h = c->h;
    c->g.pitch = c->pitch;
    c->g.nstrips = (c->ny + kStrip - 1) / kStrip;
    c->g.tiles_x = (c->nx + kWarpCols - 1) / kWarpCols;
    c->g.tiles_y = (c->g.nstrips + kBlockWarps - 1) / kBlockWarps;
    c->g.tiles = c->g.tiles_x * c->g.tiles_y;
    c->first = true;
    c->dt = cfg->dtinit;
    c->inner_fuse = kInnerFuseDefault;
    c->inner_seg = kInnerSegDefault;
    c->inner_fold_rrn = false;  // measured slower on GB300: its FP64 work lands in an issue-bound pass
    c->warm_history = 8;  // measured: 6133 against 6283 iterations over 12 timesteps of 8192^2 with 4
    c->warm_projection = TL_WARM_PROJ_ENERGY;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    c->sms = sms > 0 ? sms : 152;
    c->grid_red = sms > 0 ? sms * 4 : 512;
    if (c->grid_red > kMaxRedBlocks) c->grid_red = kMaxRedBlocks;

    int rc;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "cudaStreamCreate");
        chunk_release(c);
        return rc;
    }
    double **fields[] = {&c->density, &c->energy0, &c->energy1, &c->u,  &c->u0,    &c->p,
                         &c->r,       &c->w,       &c->z,       &c->mi, &c->kx,    &c->ky,
                         &c->sd,      &c->rtemp,   &c->utemp,   &c->r_store, &c->cp, &c->bfp,
                         &c->volume,  &c->un,    &c->diag};
    for (double **f : fields) {
        void *p;
        if ((rc = dalloc(c, &p, c->alloc_elems * sizeof(double)))) {
            chunk_release(c);
            return rc;
        }
        *f = (double *)p + c->lead;
    }
    double **mesh[] = {&c->vertexx, &c->vertexy, &c->cellx, &c->celly, &c->celldx, &c->celldy};
    size_t mlen = (size_t)(c->nx > c->ny ? c->nx : c->ny) + 2 * c->h + 2;
    for (double **f : mesh) {
        void *p;
        if ((rc = dalloc(c, &p, mlen * sizeof(double)))) {
            chunk_release(c);
            return rc;
        }
        *f = (double *)p;
    }
    void *p;
    if ((rc = dalloc(c, &p, sizeof(double) * kMaxRedBlocks * 4))) { chunk_release(c); return rc; }
    c->partials = (double *)p;
    if ((rc = dalloc(c, &p, 256))) { chunk_release(c); return rc; }
    c->counter = (unsigned int *)p;
    if ((rc = dalloc(c, &p, sizeof(DevScalars)))) { chunk_release(c); return rc; }
    c->sc = (DevScalars *)p;
    size_t nit = (size_t)cfg->max_iters + 4;
    if ((rc = dalloc(c, &p, nit * sizeof(double)))) { chunk_release(c); return rc; }
    c->cg_alphas = (double *)p;
    if ((rc = dalloc(c, &p, nit * sizeof(double)))) { chunk_release(c); return rc; }
    c->cg_betas = (double *)p;
    c->n_coefs_cap = (int)(nit > (size_t)cfg->ppcg_inner_steps + 4 ? nit : (size_t)cfg->ppcg_inner_steps + 4);
    if ((rc = dalloc(c, &p, (size_t)c->n_coefs_cap * sizeof(double)))) { chunk_release(c); return rc; }
    c->ch_alphas = (double *)p;
    if ((rc = dalloc(c, &p, (size_t)c->n_coefs_cap * sizeof(double)))) { chunk_release(c); return rc; }
    c->ch_betas = (double *)p;
    e = cudaHostAlloc((void **)&c->sc_host, 3 * sizeof(DevScalars), cudaHostAllocDefault);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "cudaHostAlloc");
        chunk_release(c);
        return rc;
    }
    memset(c->sc_host, 0, 3 * sizeof(DevScalars));
    c->poll_host = c->sc_host + 1;
    for (int k = 0; k < 2; ++k) {
        e = cudaEventCreateWithFlags(&c->poll_ev[k], cudaEventDisableTiming);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "cudaEventCreate");
            chunk_release(c);
            return rc;
        }
    }
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "chunk init");
        chunk_release(c);
        return rc;
    }
    *out = c;
    return TL_OK;
}

int chunk_sync_scalars(Chunk *c) {
    TL_CUDA(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, c->stream));
    TL_CUDA(cudaStreamSynchronize(c->stream));
    return TL_OK;
}

int chunk_push_scalars(Chunk *c) {
    TL_CUDA(cudaMemcpyAsync(c->sc, c->sc_host, sizeof(DevScalars), cudaMemcpyHostToDevice, c->stream));
    return TL_OK;
}

// initialise_chunk_kernel.cuknl:3-70 on the host (one-dimensional arrays),
// volume = dx*dy on the device
int chunk_initialise_mesh(Chunk *c, double xmin, double ymin, double dx, double dy) {
    const int h = c->h;
    const int nvx = c->nx + 2 * h + 1, nvy = c->ny + 2 * h + 1;
    c->h_vertexx.assign(nvx + 1, 0.0);
    c->h_vertexy.assign(nvy + 1, 0.0);
    c->h_cellx.assign(nvx, 0.0);
    c->h_celly.assign(nvy, 0.0);
    std::vector<double> cdx(nvx, dx), cdy(nvy, dy);
    for (int col = 0; col < nvx; ++col) {
        c->h_vertexx[col] = xmin + dx * (double)(col - h);
        double plus = xmin + dx * (double)(col - h + 1);
        c->h_cellx[col] = 0.5 * (c->h_vertexx[col] + plus);
    }
    for (int row = 0; row < nvy; ++row) {
        c->h_vertexy[row] = ymin + dy * (double)(row - h);
        double plus = ymin + dy * (double)(row - h + 1);
        c->h_celly[row] = 0.5 * (c->h_vertexy[row] + plus);
    }
    c->dx = dx;
    c->dy = dy;
    TL_CUDA(cudaMemcpyAsync(c->vertexx, c->h_vertexx.data(), nvx * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    TL_CUDA(cudaMemcpyAsync(c->vertexy, c->h_vertexy.data(), nvy * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    TL_CUDA(cudaMemcpyAsync(c->cellx, c->h_cellx.data(), nvx * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    TL_CUDA(cudaMemcpyAsync(c->celly, c->h_celly.data(), nvy * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    TL_CUDA(cudaMemcpyAsync(c->celldx, cdx.data(), nvx * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    TL_CUDA(cudaMemcpyAsync(c->celldy, cdy.data(), nvy * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int rc = launch_fill(c, c->volume, dx * dy);
    if (rc) return rc;
    TL_CUDA(cudaStreamSynchronize(c->stream));
    return TL_OK;
}

int chunk_update_halo(Chunk *c, const int *fields, int depth) {
    if (!c->cfg.reflective_boundary) return TL_OK;
    double *f[7] = {c->density, c->energy0, c->energy1, c->u, c->p, c->sd, c->r};
    for (int k = 0; k < 7; ++k)
        if (fields[k]) {
            int rc = launch_reflect(c, f[k], depth);
            if (rc) return rc;
        }
    return TL_OK;
}

// tea_leaf_kernel_cuda.cu:89-104, with the buffer sized once for the
// largest request (the reference sizes it for the first call only)
int chunk_upload_coefs(Chunk *c, const double *a, const double *b, int n) {
    if (n < 0) return TL_OK;
    if (n > c->n_coefs_cap) {
        double *na = nullptr, *nb = nullptr;
        TL_CUDA(device_malloc((void **)&na, (size_t)n * sizeof(double)));
        c->allocations.push_back(na);  // freed with the chunk even if the next one fails
        TL_CUDA(device_malloc((void **)&nb, (size_t)n * sizeof(double)));
        c->allocations.push_back(nb);
        c->ch_alphas = na;
        c->ch_betas = nb;
        c->n_coefs_cap = n;
        drop_graphs(c);  // graphs captured the old pointers
    }
    if (n == 0) return TL_OK;
    TL_CUDA(cudaMemcpyAsync(c->ch_alphas, a, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    TL_CUDA(cudaMemcpyAsync(c->ch_betas, b, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    TL_CUDA(cudaStreamSynchronize(c->stream));
    return TL_OK;
}

// ------------------------------------------------------------ profiling

int prof_begin(Chunk *c, const char *name, int *slot) {
    int kid = -1;
    for (size_t k = 0; k < c->prof_names.size(); ++k)
        if (c->prof_names[k] == name || strcmp(c->prof_names[k], name) == 0) {
            kid = (int)k;
            break;
        }
    if (kid < 0) {
        kid = (int)c->prof_names.size();
        c->prof_names.push_back(name);
        c->prof_launches.push_back(0);
        c->prof_ms.push_back(0.0);
    }
    std::pair<cudaEvent_t, cudaEvent_t> ev;
    if (!c->ev_pool.empty()) {
        ev = c->ev_pool.back();
        c->ev_pool.pop_back();
    } else {
        if (cudaEventCreate(&ev.first) != cudaSuccess) return -1;
        if (cudaEventCreate(&ev.second) != cudaSuccess) return -1;
    }
    cudaEventRecord(ev.first, c->stream);
    c->ev_pending.push_back({kid, ev});
    *slot = (int)c->ev_pending.size() - 1;
    return 0;
}

void prof_end(Chunk *c, int slot) { cudaEventRecord(c->ev_pending[slot].second.second, c->stream); }

int prof_flush(Chunk *c) {
    if (c->ev_pending.empty()) return TL_OK;
    TL_CUDA(cudaStreamSynchronize(c->stream));
    for (auto &p : c->ev_pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
            c->prof_ms[p.first] += ms;
            c->prof_launches[p.first] += 1;
        }
        c->ev_pool.push_back(p.second);
    }
    c->ev_pending.clear();
    return TL_OK;
}

static int field_summary(Chunk *c, double *vol, double *mass, double *ie, double *temp) {
    int rc = launch_field_summary(c);
    if (rc) return rc;
    if ((rc = chunk_sync_scalars(c))) return rc;
    if (vol) *vol = c->sc_host->sum[0];
    if (mass) *mass = c->sc_host->sum[1];
    if (ie) *ie = c->sc_host->sum[2];
    if (temp) *temp = c->sc_host->sum[3];
    return TL_OK;
}

void drop_graphs(Chunk *c) {
    for (cudaGraphExec_t &g : c->graphs)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

// Host copies of a field: from page-locked, mapped host memory a kernel
// reads (or writes) the host array directly and re-pitches it in the same
// pass; from other host memory the field moves as one contiguous block
// through a device staging buffer (rows x (nx + 2h), the host layout) that
// a kernel re-pitches.  (A pitched 2-D copy moves one short row at a time
// and runs far below the host link's bandwidth.)
// to_pitched: dst[r * pitch + c] = src[r * w + c]; else the reverse
static __global__ void k_repitch(double *__restrict__ dst, const double *__restrict__ src, int w, int pitch,
                          int rows, bool to_pitched) {
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int64_t dense = (int64_t)r * w, pitched = (int64_t)r * pitch;
        for (int col = threadIdx.x; col < w; col += blockDim.x) {
            if (to_pitched) dst[pitched + col] = src[dense + col];
            else dst[dense + col] = src[pitched + col];
        }
    }
}

// the device address of page-locked, mapped host memory (cudaHostAlloc /
// cudaHostRegister), or nullptr for any other host pointer: a kernel then
// moves the field between HBM and the host in one pass, re-pitching as it
// goes, instead of a DMA copy through the staging buffer
static void *mapped_host(const void *host) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();  // an unregistered pointer is not an error here
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

static int stage_buffer(Chunk *c, double **out) {
    if (!c->stage) {
        void *p;
        int rc = dalloc(c, &p, (size_t)(c->nx + 2 * c->h) * (size_t)c->rows * sizeof(double));
        if (rc) return rc;
        c->stage = (double *)p;
    }
    *out = c->stage;
    return TL_OK;
}

}  // namespace tl

using namespace tl;

struct tl_chunk {
    Chunk *c;
};

static tl_chunk g_default = {nullptr};

static int field_arg(tl_chunk_t *ch, int field, const void *host, const char *what, double **f) {
    if (!ch || !ch->c || !host) {
        set_error("%s: bad argument", what);
        return TL_ERR_ARG;
    }
    *f = field_ptr(ch->c, field);
    if (!*f) {
        set_error("%s: unknown field %d", what, field);
        return TL_ERR_ARG;
    }
    return TL_OK;
}


extern "C" {

const char *tl_last_error(void) { return g_err; }
void tl_clear_error(void) { g_err[0] = '\0'; }
const char *tl_version(void) { return "tealeaf_gb300 1.0 (sm_103a)"; }

int tl_test_fail_alloc(int nth) {
    if (nth < 0) {
        set_error("tl_test_fail_alloc: nth must be >= 0");
        return TL_ERR_ARG;
    }
    g_fail_alloc_countdown.store(nth);
    return TL_OK;
}

long long tl_sizeof(int which) {
    switch (which) {
    case 0: return (long long)sizeof(tl_config_t);
    case 1: return (long long)sizeof(tl_solve_info_t);
    case 2: return (long long)sizeof(tl_step_record_t);
    case 3: return (long long)sizeof(tl_run_options_t);
    case 4: return (long long)sizeof(tl_run_result_t);
    case 5: return (long long)sizeof(tl_state_t);
    default: return -1;
    }
}

int tl_chunk_create(const tl_config_t *cfg, tl_chunk_t **out) {
    if (!cfg || !out) {
        set_error("tl_chunk_create: null argument");
        return TL_ERR_ARG;
    }
    Chunk *c;
    int rc = chunk_alloc(cfg, &c);
    if (rc) return rc;
    tl_chunk_t *h = new tl_chunk{c};
    *out = h;
    return TL_OK;
}

int tl_chunk_destroy(tl_chunk_t *ch) {
    if (!ch) return TL_OK;
    chunk_release(ch->c);
    if (ch != &g_default) delete ch;
    else g_default.c = nullptr;
    return TL_OK;
}

tl_chunk_t *tl_default_chunk(void) { return g_default.c ? &g_default : nullptr; }

int tl_start(tl_chunk_t *ch, double *vol, double *mass, double *ie, double *temp) {
    if (!ch || !ch->c) {
        set_error("tl_start: no chunk");
        return TL_ERR_STATE;
    }
    Chunk *c = ch->c;
    const tl_config_t &cf = c->cfg;
    // initialise_chunk.f90:33-40
    double dx = (cf.xmax - cf.xmin) / (double)(float)cf.x_cells;
    double dy = (cf.ymax - cf.ymin) / (double)(float)cf.y_cells;
    int rc = chunk_initialise_mesh(c, cf.xmin, cf.ymin, dx, dy);
    if (rc) return rc;
    // generate_chunk.f90 / generate_chunk_kernel_cuda.cu:50-110
    tl_state_t *sdev = nullptr;
    TL_CUDA(device_malloc((void **)&sdev, sizeof(tl_state_t) * (cf.nstates > 0 ? cf.nstates : 1)));
    cudaMemcpyAsync(sdev, cf.states, sizeof(tl_state_t) * cf.nstates, cudaMemcpyHostToDevice, c->stream);
    rc = launch_generate(c, cf.nstates, sdev);
    cudaStreamSynchronize(c->stream);
    cudaFree(sdev);
    if (rc) return rc;
    // start.f90:88-105: halo of density/energy, then energy1 = energy0
    int fl[7] = {1, 1, 1, 0, 0, 0, 0};
    if ((rc = chunk_update_halo(c, fl, c->h))) return rc;
    if ((rc = launch_set_field(c))) return rc;
    c->dt = cf.dtinit;
    // a (re)start begins a fresh run: the tea_solve.f90 SAVE state (first
    // solve, eigenvalue estimates) and the warm start's u^(n-1) are reset
    c->first = true;
    c->eigmin = c->eigmax = c->theta = c->cn = 0.0;
    warm_reset(c);
    return field_summary(c, vol, mass, ie, temp);
}

int tl_timestep(tl_chunk_t *ch, tl_solve_info_t *info) {
    if (!ch || !ch->c || !info) {
        set_error("tl_timestep: no chunk");
        return TL_ERR_STATE;
    }
    const tl_config_t &cf = ch->c->cfg;
    if (cf.precision == TL_PRECISION_MIXED) {
        if (cf.solver == TL_SOLVER_PPCG) {
            // FP64 flexible outer iteration, FP32 polynomial preconditioner
            if (cf.reflective_boundary) {
                set_error("tl_precision mixed does not support reflective_boundary");
                return TL_ERR_ARG;
            }
            return solve_timestep(ch->c, info);
        }
        return solve_timestep_mixed(ch->c, info);
    }
    return solve_timestep(ch->c, info);
}

int tl_field_summary(tl_chunk_t *ch, double *vol, double *mass, double *ie, double *temp) {
    if (!ch || !ch->c) {
        set_error("tl_field_summary: no chunk");
        return TL_ERR_STATE;
    }
    return field_summary(ch->c, vol, mass, ie, temp);
}


int tl_get_field(tl_chunk_t *ch, int field, double *host) {
    double *f;
    int rc = field_arg(ch, field, host, "tl_get_field", &f);
    if (rc) return rc;
    Chunk *c = ch->c;
    const int w = c->nx + 2 * c->h;
    const size_t bytes = (size_t)w * (size_t)c->rows * sizeof(double);
    double *mapped = (double *)mapped_host(host);
    if (w == c->pitch) {
        TL_CUDA(cudaMemcpyAsync(host, f, bytes, cudaMemcpyDeviceToHost, c->stream));
    } else if (mapped) {
        k_repitch<<<c->sms * 8, 256, 0, c->stream>>>(mapped, f, w, c->pitch, c->rows, false);
        TL_CUDA(cudaGetLastError());
        c->launches++;
    } else {
        double *st;
        if ((rc = stage_buffer(c, &st))) return rc;
        k_repitch<<<c->sms * 8, 256, 0, c->stream>>>(st, f, w, c->pitch, c->rows, false);
        TL_CUDA(cudaGetLastError());
        c->launches++;
        TL_CUDA(cudaMemcpyAsync(host, st, bytes, cudaMemcpyDeviceToHost, c->stream));
    }
    TL_CUDA(cudaStreamSynchronize(c->stream));
    return TL_OK;
}

int tl_set_field(tl_chunk_t *ch, int field, const double *host) {
    double *f;
    int rc = field_arg(ch, field, host, "tl_set_field", &f);
    if (rc) return rc;
    Chunk *c = ch->c;
    const int w = c->nx + 2 * c->h;
    const size_t bytes = (size_t)w * (size_t)c->rows * sizeof(double);
    const double *mapped = (const double *)mapped_host(host);
    if (w == c->pitch) {
        TL_CUDA(cudaMemcpyAsync(f, host, bytes, cudaMemcpyHostToDevice, c->stream));
    } else if (mapped) {
        k_repitch<<<c->sms * 8, 256, 0, c->stream>>>(f, mapped, w, c->pitch, c->rows, true);
        TL_CUDA(cudaGetLastError());
        c->launches++;
    } else {
        double *st;
        if ((rc = stage_buffer(c, &st))) return rc;
        TL_CUDA(cudaMemcpyAsync(st, host, bytes, cudaMemcpyHostToDevice, c->stream));
        k_repitch<<<c->sms * 8, 256, 0, c->stream>>>(f, st, w, c->pitch, c->rows, true);
        TL_CUDA(cudaGetLastError());
        c->launches++;
    }
    // the caller may reuse its buffer once this returns
    TL_CUDA(cudaStreamSynchronize(c->stream));
    return TL_OK;
}

int tl_set_dt(tl_chunk_t *ch, double dt) {
    if (!ch || !ch->c) {
        set_error("tl_set_dt: no chunk");
        return TL_ERR_STATE;
    }
    ch->c->dt = dt;
    return TL_OK;
}

long long tl_kernel_launches(tl_chunk_t *ch) { return (ch && ch->c) ? ch->c->launches : 0; }

void *tl_chunk_stream(tl_chunk_t *ch) { return (ch && ch->c) ? (void *)ch->c->stream : nullptr; }

int tl_set_warm_start_model(tl_chunk_t *ch, const float *params, long long n) {
    if (!ch || !ch->c || !params) {
        set_error("tl_set_warm_start_model: bad argument");
        return TL_ERR_ARG;
    }
    return warm_set_model(ch->c, params, n);
}

int tl_set_warm_start_options(tl_chunk_t *ch, int history, int projection) {
    if (!ch || !ch->c) {
        set_error("tl_set_warm_start_options: no chunk");
        return TL_ERR_STATE;
    }
    return warm_set_options(ch->c, history, projection);
}

int tl_warm_start_features(tl_chunk_t *ch, float *dst) {
    if (!ch || !ch->c || !dst) {
        set_error("tl_warm_start_features: bad argument");
        return TL_ERR_ARG;
    }
    return warm_features(ch->c, dst);
}

int tl_set_inner_fusion(tl_chunk_t *ch, int steps, int seg_strips, int fold_rrn) {
    if (!ch || !ch->c) {
        set_error("tl_set_inner_fusion: no chunk");
        return TL_ERR_STATE;
    }
    if (steps < 1 || steps > kFusedMax || seg_strips < 0) {
        set_error("tl_set_inner_fusion: steps must be 1..%d and seg_strips >= 0 (got %d, %d)", kFusedMax, steps,
                  seg_strips);
        return TL_ERR_ARG;
    }
    Chunk *c = ch->c;
    if (c->inner_fuse != steps || c->inner_seg != seg_strips || c->inner_fold_rrn != (fold_rrn != 0))
        drop_graphs(c);
    c->inner_fuse = steps;
    c->inner_seg = seg_strips;
    c->inner_fold_rrn = fold_rrn != 0;
    return TL_OK;
}

int tl_set_profiling(tl_chunk_t *ch, int on) {
    if (!ch || !ch->c) {
        set_error("tl_set_profiling: no chunk");
        return TL_ERR_STATE;
    }
    int rc = prof_flush(ch->c);
    ch->c->profiling = on != 0;
    return rc;
}

int tl_profile_reset(tl_chunk_t *ch) {
    if (!ch || !ch->c) return TL_ERR_STATE;
    int rc = prof_flush(ch->c);
    for (auto &v : ch->c->prof_ms) v = 0.0;
    for (auto &v : ch->c->prof_launches) v = 0;
    return rc;
}

int tl_profile_read(tl_chunk_t *ch, int idx, const char **name, long long *launches, double *ms) {
    if (!ch || !ch->c) return TL_ERR_STATE;
    Chunk *c = ch->c;
    int rc = prof_flush(c);
    if (rc) return rc;
    if (idx < 0 || idx >= (int)c->prof_names.size()) return TL_ERR_ARG;
    if (name) *name = c->prof_names[idx];
    if (launches) *launches = c->prof_launches[idx];
    if (ms) *ms = c->prof_ms[idx];
    return TL_OK;
}

}  // extern "C"

// the process-wide chunk of the reference-named entry points
namespace tl {
int default_chunk_replace(const tl_config_t *cfg);
}
extern "C" int tl_default_chunk_init(const tl_config_t *cfg) {
    if (!cfg) {
        set_error("tl_default_chunk_init: null config");
        return TL_ERR_ARG;
    }
    return tl::default_chunk_replace(cfg);
}
namespace tl {
int default_chunk_replace(const tl_config_t *cfg) {
    if (g_default.c) {
        chunk_release(g_default.c);
        g_default.c = nullptr;
    }
    Chunk *c;
    int rc = chunk_alloc(cfg, &c);
    if (rc) return rc;
    g_default.c = c;
    return TL_OK;
}
Chunk *default_chunk() { return g_default.c; }
}  // namespace tl
