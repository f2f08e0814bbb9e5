// pf_api.cu -- the C ABI of libpfstep: the drop-in GPU_* plug-in and the
// full-step pf_* context (state resident in HBM, kernels on one stream).
//
// Step orchestration follows phase_field::Update (zhubq/PhaseField,
// C++-openmp-cuda/src/phase_field.cpp:243-305): evaluate the step's parameters
// at the current time and advance time by pfm_dt (Update_parameter, :307-315),
// one phase sweep into the second id/phi buffer and swap (:252-260), then
// n_sub = max(ceil(pfm_dt/diff_dt),1) diffusion sub-steps of pfm_dt/n_sub,
// swapping the concentration buffers after each (:408-418).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include "pf_dev.cuh"
#include "pf_host.h"
#include "pf_kernels.h"
#include "pf_output.h"

static int pf_cuda_fail(cudaError_t e) {
    return pf_fail(PF_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
}

// ===========================================================================
// 1. Drop-in for gpu_solver.h (module state, single host thread, like the
//    reference's statics in gpu_solver.cpp:13-18).
// ===========================================================================
namespace {
struct DropIn {
    int x = 0, y = 0, z = 0;
    double *phase = nullptr, *C = nullptr, *conc[2] = {nullptr, nullptr};
    double *links = nullptr;  // flux weights of the forward links (k_links_f64)
    double *tpart = nullptr;  // partition sums of the fixed phase fractions
    bool ready = false;
} g_drop;

void dropin_free() {
    cudaFree(g_drop.phase);
    cudaFree(g_drop.C);
    cudaFree(g_drop.conc[0]);
    cudaFree(g_drop.conc[1]);
    cudaFree(g_drop.links);
    cudaFree(g_drop.tpart);
    g_drop = DropIn();
}
}  // namespace

extern "C" int GPU_Init(const int x, const int y, const int z) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return 0;
    }
    if (cudaSetDevice(0) != cudaSuccess) return 0;
    if (x < 1 || y < 1 || z < 1) return 0;
    if (g_drop.ready) dropin_free();
    const size_t N = (size_t)x * y * z;
    size_t freeb = 0, total = 0;
    cudaMemGetInfo(&freeb, &total);
    if (N * sizeof(double) * 25 > freeb) return 0;
    if (cudaMalloc(&g_drop.phase, 3 * N * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&g_drop.links, 9 * N * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&g_drop.tpart, 6 * N * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&g_drop.C, N * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&g_drop.conc[0], 3 * N * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&g_drop.conc[1], 3 * N * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        dropin_free();
        return 0;
    }
    g_drop.x = x; g_drop.y = y; g_drop.z = z;
    g_drop.ready = true;
    return 1;
}

extern "C" void GPU_Diffusion_solver(double *hdiffusivity, double *hpartition_k, double *hpartition_c,
                                     double *hvalue_phase, double *htotal_conc, int x, int y, int z,
                                     double dt, double dx) {
    if (!g_drop.ready || x != g_drop.x || y != g_drop.y || z != g_drop.z) {
        if (!GPU_Init(x, y, z)) {
            pf_fail(PF_ERR_NODEV, "GPU_Diffusion_solver: GPU_Init failed");
            return;
        }
    }
    const long long N = (long long)x * y * z;
    pf_step_params P;
    std::memset(&P, 0, sizeof(P));
    P.ix = x; P.iy = y; P.iz = z; P.N = N; P.nsol = 1;
    for (int p = 0; p < 3; p++) P.D[0][p] = hdiffusivity[p];
    for (int e = 0; e < 9; e++) {
        P.k[0][e] = hpartition_k[e];
        P.c[0][e] = hpartition_c[e];
    }
    // gpu_solver.cpp:93-94, 206-209 (0.2f kept: it decides num_loop).
    const int dims = z > 1 ? 3 : 2;
    double max_diff = hdiffusivity[0];
    for (int p = 1; p < 3; p++)
        if (hdiffusivity[p] > max_diff) max_diff = hdiffusivity[p];
    const double del_t = dx * dx / max_diff / dims * 0.2f;
    const int num_loop = (int)std::ceil(dt / del_t);
    const double dt_dxdx = dt / num_loop / (dx * dx);
    cudaStream_t s = 0;
    cudaMemcpy(g_drop.phase, hvalue_phase, 3 * N * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(g_drop.C, htotal_conc, N * sizeof(double), cudaMemcpyHostToDevice);
    pf_launch_partition_f64(P, g_drop.phase, g_drop.C, g_drop.conc[0], s);
    pf_launch_links_f64(P, 6, g_drop.phase, g_drop.links, g_drop.tpart, s);  // phases fixed for the whole call
    int a = 0;
    for (int it = 1; it <= num_loop; it++) {
        pf_launch_diffuse_f64(P, 6, dt_dxdx, g_drop.links, g_drop.tpart, g_drop.conc[a], g_drop.conc[1 - a],
                              g_drop.C, s);
        a = 1 - a;
    }
    cudaError_t e = cudaMemcpy(htotal_conc, g_drop.C, N * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) pf_cuda_fail(e);
}

extern "C" void GPU_Cleanup(void) {
    if (g_drop.ready) dropin_free();
}

// ===========================================================================
// 2. Full-step context.
// ===========================================================================
struct pf_ctx {
    pf_model model;
    int prec = PF_PREC_FP64;
    long long N = 0;
    int nsol = 1;
    double time = 0.;
    bool have_state = false;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // FP64 reference layout
    int *ids[2] = {nullptr, nullptr};
    double *phi[2] = {nullptr, nullptr};
    double *phase = nullptr;
    double *conc[2] = {nullptr, nullptr};
    double *C = nullptr;
    double *avg = nullptr;  // interface-averaged concentrations (models with avg_carbon or coherent)
    double *links = nullptr;  // flux weights of the forward links, refreshed after each phase sweep
    double *tpart = nullptr;  // partition sums of the same phase fractions
    unsigned char *coh_flags = nullptr;  // Has_ferrite / Rex_intf per cell (models with coherent)
    int *coh = nullptr;                  // coherent partners, 2 per austenite grain
    int n_coh = 0;
    int cur = 0, curc = 0;
    // FP32 compact layout
    ushort4 *gid[2] = {nullptr, nullptr};
    float4 *phi32[2] = {nullptr, nullptr};
    float *phase32 = nullptr;
    float2 *sol[2] = {nullptr, nullptr};
    int curs = 0;
    pf_f32_map map{};
    int *d_span = nullptr;
    unsigned int *d_trunc = nullptr;
    unsigned int *rest = nullptr;        // phase sweep: cells with more than four stencil grains
    unsigned int *rest_count = nullptr;
    pf_out *out = nullptr;               // asynchronous binary microstructure writer
    long long truncated = 0;
    // Reference-layout (FP64) staging buffers of the FP32C upload/download,
    // allocated on first use and kept until pf_destroy, so repeated uploads
    // and downloads allocate nothing.
    int *st_ids = nullptr;
    double *st_phi = nullptr, *st_phase = nullptr, *st_C = nullptr, *st_conc = nullptr;
    // reductions
    double *partials = nullptr;
    int red_blocks = 0;
    double *d_red = nullptr;
    double *h_red = nullptr;  // pinned
    // per-step bookkeeping
    pf_step_params last{};
    bool have_last = false;
    double last_temperature_written = 0.;
    int micro_count = 0;
    // kernel timing
    bool ktiming = false;
    std::vector<cudaEvent_t> ev_free;
    struct Pending { cudaEvent_t a, b; int kind; };
    std::vector<Pending> pending;
    double ktime[2] = {0., 0.};
    long long kcount[2] = {0, 0};
    // graphs
    bool use_graph = false;
    cudaGraphExec_t gexec = nullptr;
    pf_step_params gparams{};
    int gphase = -1;
    // diffusion tile shape chosen by pf_autotune (FP32C)
    pf_diff_cfg diff_cfg{8, 16, 0};
    bool diff_cfg_valid = false;
    float diff_cfg_ms = 0.f;
};

namespace {

cudaEvent_t ev_get(pf_ctx *c) {
    if (!c->ev_free.empty()) {
        cudaEvent_t e = c->ev_free.back();
        c->ev_free.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

int collect_times(pf_ctx *c) {
    if (c->pending.empty()) return PF_OK;
    PF_CUDA_OK(cudaStreamSynchronize(c->stream));
    for (auto &p : c->pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        c->ktime[p.kind] += ms;
        c->kcount[p.kind] += 1;
        c->ev_free.push_back(p.a);
        c->ev_free.push_back(p.b);
    }
    c->pending.clear();
    return PF_OK;
}

template <class F>
cudaError_t timed(pf_ctx *c, int kind, F launch) {
    if (!c->ktiming) return launch();
    cudaEvent_t a = ev_get(c), b = ev_get(c);
    cudaEventRecord(a, c->stream);
    cudaError_t e = launch();
    cudaEventRecord(b, c->stream);
    c->pending.push_back({a, b, kind});
    if (c->pending.size() > 4096) collect_times(c);
    return e;
}

void free_all(pf_ctx *c) {
    pf_out_destroy(c->out);
    c->out = nullptr;
    for (int i = 0; i < 2; i++) {
        cudaFree(c->ids[i]); cudaFree(c->phi[i]); cudaFree(c->conc[i]);
        cudaFree(c->gid[i]); cudaFree(c->phi32[i]); cudaFree(c->sol[i]);
    }
    cudaFree(c->phase); cudaFree(c->C); cudaFree(c->avg); cudaFree(c->links); cudaFree(c->tpart); cudaFree(c->coh_flags); cudaFree(c->coh); cudaFree(c->phase32);
    cudaFree(c->d_span); cudaFree(c->d_trunc); cudaFree(c->rest); cudaFree(c->rest_count);
    cudaFree(c->st_ids); cudaFree(c->st_phi); cudaFree(c->st_phase); cudaFree(c->st_C); cudaFree(c->st_conc);
    cudaFree(c->partials); cudaFree(c->d_red);
    if (c->h_red) cudaFreeHost(c->h_red);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    for (auto &p : c->pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : c->ev_free) cudaEventDestroy(e);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
}

// Launch one full step with parameters P (no parameter evaluation, no time
// update).  Buffer roles advance.
cudaError_t launch_step(pf_ctx *c, const pf_step_params &P) {
    cudaError_t e = cudaSuccess;
    if (c->prec == PF_PREC_FP64) {
        const int a = c->cur;
        e = timed(c, 0, [&] {
            return pf_launch_phase_f64(P, c->ids[a], c->phi[a], c->ids[1 - a], c->phi[1 - a], c->phase,
                                       c->conc[c->curc], c->C, c->avg, c->coh_flags, c->coh, c->n_coh,
                                       c->stream);
        });
        if (e != cudaSuccess) return e;
        c->cur = 1 - a;
        e = timed(c, 1, [&] { return pf_launch_links_f64(P, P.nnb, c->phase, c->links, c->tpart, c->stream); });
        if (e != cudaSuccess) return e;
        for (int it = 0; it < P.n_sub; it++) {
            const int b = c->curc;
            e = timed(c, 1, [&] {
                return pf_launch_diffuse_f64(P, P.nnb, P.coef_diff, c->links, c->tpart, c->conc[b], c->conc[1 - b],
                                             c->C, c->stream);
            });
            if (e != cudaSuccess) return e;
            c->curc = 1 - b;
        }
    } else {
        pf_f32_params F;
        pf_fold_f32(P, c->map.off[2], c->map.off[3], F);
        const int a = c->cur;
        e = timed(c, 0, [&] {
            return pf_launch_phase_f32(F, c->gid[a], c->phi32[a], c->gid[1 - a], c->phi32[1 - a], c->phase32,
                                       c->sol[c->curs], c->rest, c->rest_count, c->stream);
        });
        if (e != cudaSuccess) return e;
        c->cur = 1 - a;
        for (int it = 0; it < P.n_sub; it++) {
            const int b = c->curs;
            e = timed(c, 1, [&] {
                return pf_launch_diffuse_f32(F, c->phase32, c->sol[b], c->sol[1 - b], c->stream, c->diff_cfg_valid ? &c->diff_cfg : nullptr);
            });
            if (e != cudaSuccess) return e;
            c->curs = 1 - b;
        }
    }
    return e;
}

// The FP32C context's reference-layout staging buffers (conc only when asked).
bool ensure_staging(pf_ctx *c, bool conc) {
    const size_t N = (size_t)c->N;
    bool ok = true;
    auto alloc = [&](void **p, size_t bytes) {
        if (ok && !*p && cudaMalloc(p, bytes) != cudaSuccess) {
            *p = nullptr;
            ok = false;
        }
    };
    alloc((void **)&c->st_ids, 6 * N * sizeof(int));
    alloc((void **)&c->st_phi, 6 * N * sizeof(double));
    alloc((void **)&c->st_phase, 3 * N * sizeof(double));
    alloc((void **)&c->st_C, N * c->nsol * sizeof(double));
    if (conc) alloc((void **)&c->st_conc, 3 * N * c->nsol * sizeof(double));
    if (!ok) cudaGetLastError();
    return ok;
}

bool same_step(const pf_step_params &a, const pf_step_params &b) {
    pf_step_params x = a, y = b;
    x.time = y.time = 0.;
    return std::memcmp(&x, &y, sizeof(x)) == 0;
}

// Buffer-role signature: graphs are captured for a fixed assignment.
int role_sig(const pf_ctx *c) { return c->cur | (c->curc << 1) | (c->curs << 2); }

}  // namespace

namespace {
// The reference-layout state in the FP32C context's staging buffers -> the
// compact layout: local id map from the grain-id spans, then the pack kernel.
int pack_staged(pf_ctx *c, const char *who) {
    int st = PF_OK;
    cudaMemsetAsync(c->d_span, 0, 8 * sizeof(int), c->stream);
    cudaMemsetAsync(c->d_trunc, 0, sizeof(unsigned int), c->stream);
    pf_launch_id_span(c->st_ids, c->N, c->d_span, c->stream);
    int span[8];
    cudaError_t e = cudaMemcpyAsync(span, c->d_span, 8 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) st = pf_cuda_fail(e);
    else if (span[4] != 0) st = pf_fail(PF_ERR_RANGE, std::string(who) + ": grain id outside 0..399999");
    else {
        c->map.off[0] = 0;
        c->map.off[1] = span[0];
        c->map.off[2] = span[0] + span[1];
        c->map.off[3] = span[0] + span[1] + span[2];
        c->map.total = c->map.off[3] + span[3];
        if (c->map.total > 65535) st = pf_fail(PF_ERR_RANGE, std::string(who) + ": more than 65535 grains");
    }
    if (st == PF_OK) {
        e = pf_launch_pack_f32(c->N, c->nsol, c->map, c->st_ids, c->st_phi, c->st_phase, c->st_C, c->gid[0],
                               c->phi32[0], c->phase32, c->sol[0], c->d_trunc, c->stream);
        unsigned int tr = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&tr, c->d_trunc, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) st = pf_cuda_fail(e);
        c->truncated = tr;
    }
    cudaStreamSynchronize(c->stream);
    return st;
}
}  // namespace

extern "C" int pf_create(const pf_model *model, int precision, pf_ctx **out) {
    if (!model || !out) return pf_fail(PF_ERR_ARG, "pf_create: null argument");
    *out = nullptr;
    if (precision != PF_PREC_FP64 && precision != PF_PREC_FP32C) return pf_fail(PF_ERR_ARG, "pf_create: bad precision");
    if (model->ix < 1 || model->iy < 1 || model->iz < 1 || model->nsol < 1 || model->nsol > 2 || model->nT < 1)
        return pf_fail(PF_ERR_ARG, "pf_create: bad model");
    if (precision == PF_PREC_FP32C && (long long)model->ix * model->iy * model->iz > 0xffffffffLL)
        return pf_fail(PF_ERR_RANGE, "pf_create: the compact FP32 path indexes cells with 32 bits");
    if (precision == PF_PREC_FP32C && (model->avg_carbon || model->drag || model->coherent))
        return pf_fail(PF_ERR_ARG,
                       "pf_create: the interface-averaged carbon, the solute drag and the coherent-grain mobility run on "
                       "the FP64 path only");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return pf_fail(PF_ERR_NODEV, "pf_create: no CUDA device");
    }
    pf_ctx *c = new pf_ctx();
    c->model = *model;
    c->prec = precision;
    c->N = (long long)model->ix * model->iy * model->iz;
    c->nsol = model->nsol;
    const size_t N = (size_t)c->N;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return pf_cuda_fail(e); }
    c->own_stream = true;
    bool ok = true;
    auto alloc = [&](void **p, size_t bytes) {
        if (ok && cudaMalloc(p, bytes) != cudaSuccess) ok = false;
    };
    if (precision == PF_PREC_FP64) {
        for (int i = 0; i < 2; i++) {
            alloc((void **)&c->ids[i], 6 * N * sizeof(int));
            alloc((void **)&c->phi[i], 6 * N * sizeof(double));
            alloc((void **)&c->conc[i], 3 * N * c->nsol * sizeof(double));
        }
        alloc((void **)&c->phase, 3 * N * sizeof(double));
        alloc((void **)&c->links, 9 * N * sizeof(double));
        alloc((void **)&c->tpart, 6 * N * c->nsol * sizeof(double));
        alloc((void **)&c->C, N * c->nsol * sizeof(double));
        if (model->avg_carbon || model->coherent) alloc((void **)&c->avg, 3 * N * sizeof(double));
        if (model->coherent) alloc((void **)&c->coh_flags, N);
    } else {
        for (int i = 0; i < 2; i++) {
            alloc((void **)&c->gid[i], N * sizeof(ushort4));
            alloc((void **)&c->phi32[i], N * sizeof(float4));
            alloc((void **)&c->sol[i], N * c->nsol * sizeof(float2));
        }
        alloc((void **)&c->phase32, 3 * N * sizeof(float));
        alloc((void **)&c->d_span, 8 * sizeof(int));
        alloc((void **)&c->d_trunc, sizeof(unsigned int));
        alloc((void **)&c->rest, N * sizeof(unsigned int));
        alloc((void **)&c->rest_count, sizeof(unsigned int));
    }
    c->red_blocks = pf_reduce_blocks(c->N);
    alloc((void **)&c->partials, (size_t)c->red_blocks * PF_RED_NOUT * sizeof(double));
    alloc((void **)&c->d_red, PF_RED_NOUT * sizeof(double));
    if (ok && cudaMallocHost((void **)&c->h_red, PF_RED_NOUT * sizeof(double)) != cudaSuccess) ok = false;
    if (!ok) {
        cudaGetLastError();
        free_all(c);
        delete c;
        return pf_fail(PF_ERR_NOMEM, "pf_create: device allocation failed");
    }
    *out = c;
    return PF_OK;
}

extern "C" int pf_destroy(pf_ctx *c) {
    if (!c) return PF_OK;
    cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
    return PF_OK;
}

extern "C" int pf_set_stream(pf_ctx *c, void *stream) {
    if (!c) return pf_fail(PF_ERR_ARG, "pf_set_stream: null context");
    PF_CUDA_OK(cudaStreamSynchronize(c->stream));
    if (c->own_stream) cudaStreamDestroy(c->stream);
    if (stream) {
        c->stream = (cudaStream_t)stream;
        c->own_stream = false;
    } else {
        PF_CUDA_OK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; c->gphase = -1; }
    return PF_OK;
}

extern "C" int pf_set_coherent_grains(pf_ctx *c, const int32_t *partners, int n_austenite) {
    if (!c) return pf_fail(PF_ERR_ARG, "pf_set_coherent_grains: null context");
    if (!c->model.coherent || c->prec != PF_PREC_FP64)
        return pf_fail(PF_ERR_ARG, "pf_set_coherent_grains: the model has no coherent-grain mobility");
    if (n_austenite < 0 || n_austenite > PF_MAXGRAIN_PER_PHASE || (n_austenite > 0 && !partners))
        return pf_fail(PF_ERR_ARG, "pf_set_coherent_grains: bad table");
    PF_CUDA_OK(cudaStreamSynchronize(c->stream));
    cudaFree(c->coh);
    c->coh = nullptr;
    c->n_coh = 0;
    if (n_austenite > 0) {
        PF_CUDA_OK(cudaMalloc((void **)&c->coh, 2 * (size_t)n_austenite * sizeof(int)));
        PF_CUDA_OK(cudaMemcpy(c->coh, partners, 2 * (size_t)n_austenite * sizeof(int), cudaMemcpyHostToDevice));
        c->n_coh = n_austenite;
    }
    // a captured step holds the old table's address
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; c->gphase = -1; }
    return PF_OK;
}

extern "C" int pf_upload_state(pf_ctx *c, const int32_t *ids, const double *phi, const double *phase,
                               const double *conc, const double *C, double time) {
    if (!c || !ids || !phi || !phase || !C) return pf_fail(PF_ERR_ARG, "pf_upload_state: null argument");
    const size_t N = (size_t)c->N;
    c->time = time;
    c->cur = c->curc = c->curs = 0;
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; c->gphase = -1; }
    pf_step_params P;
    pf_compute_params(c->model, time, P);
    if (c->prec == PF_PREC_FP64) {
        PF_CUDA_OK(cudaMemcpyAsync(c->ids[0], ids, 6 * N * sizeof(int), cudaMemcpyHostToDevice, c->stream));
        PF_CUDA_OK(cudaMemcpyAsync(c->phi[0], phi, 6 * N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        PF_CUDA_OK(cudaMemcpyAsync(c->phase, phase, 3 * N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        PF_CUDA_OK(cudaMemcpyAsync(c->C, C, N * c->nsol * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        if (conc)
            PF_CUDA_OK(cudaMemcpyAsync(c->conc[0], conc, 3 * N * c->nsol * sizeof(double), cudaMemcpyHostToDevice,
                                       c->stream));
        else
            PF_CUDA_OK(pf_launch_partition_f64(P, c->phase, c->C, c->conc[0], c->stream));
    } else {
        // The reference layout is staged in the context's FP64 buffers and
        // packed on the device.
        if (!ensure_staging(c, false)) return pf_fail(PF_ERR_NOMEM, "pf_upload_state: staging allocation failed");
        cudaMemcpyAsync(c->st_ids, ids, 6 * N * sizeof(int), cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(c->st_phi, phi, 6 * N * sizeof(double), cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(c->st_phase, phase, 3 * N * sizeof(double), cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(c->st_C, C, N * c->nsol * sizeof(double), cudaMemcpyHostToDevice, c->stream);
        const int st = pack_staged(c, "pf_upload_state");
        if (st != PF_OK) return st;
    }
    c->have_state = true;
    c->have_last = false;
    return PF_OK;
}

extern "C" int pf_download_state(pf_ctx *c, int32_t *ids, double *phi, double *phase, double *conc, double *C,
                                 double *time) {
    if (!c || !c->have_state) return pf_fail(PF_ERR_ARG, "pf_download_state: no state");
    const size_t N = (size_t)c->N;
    if (time) *time = c->time;
    if (c->prec == PF_PREC_FP64) {
        if (ids) PF_CUDA_OK(cudaMemcpyAsync(ids, c->ids[c->cur], 6 * N * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        if (phi) PF_CUDA_OK(cudaMemcpyAsync(phi, c->phi[c->cur], 6 * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        if (phase) PF_CUDA_OK(cudaMemcpyAsync(phase, c->phase, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        if (conc)
            PF_CUDA_OK(cudaMemcpyAsync(conc, c->conc[c->curc], 3 * N * c->nsol * sizeof(double), cudaMemcpyDeviceToHost,
                                       c->stream));
        if (C) PF_CUDA_OK(cudaMemcpyAsync(C, c->C, N * c->nsol * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        PF_CUDA_OK(cudaStreamSynchronize(c->stream));
        return PF_OK;
    }
    int st = PF_OK;
    if (!ensure_staging(c, conc != nullptr)) {
        st = pf_fail(PF_ERR_NOMEM, "pf_download_state: staging allocation failed");
    } else {
        int *d_ids = c->st_ids;
        double *d_phi = c->st_phi, *d_phase = c->st_phase, *d_C = c->st_C;
        double *d_conc = conc ? c->st_conc : nullptr;
        pf_step_params P;
        pf_compute_params(c->model, c->time, P);
        cudaError_t e = pf_launch_unpack_f32(P, c->map, c->gid[c->cur], c->phi32[c->cur], c->phase32, c->sol[c->curs],
                                             d_ids, d_phi, d_phase, d_conc, d_C, c->stream);
        if (e == cudaSuccess && ids) e = cudaMemcpyAsync(ids, d_ids, 6 * N * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && phi) e = cudaMemcpyAsync(phi, d_phi, 6 * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && phase)
            e = cudaMemcpyAsync(phase, d_phase, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && conc)
            e = cudaMemcpyAsync(conc, d_conc, 3 * N * c->nsol * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && C) e = cudaMemcpyAsync(C, d_C, N * c->nsol * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) st = pf_cuda_fail(e);
    }
    cudaStreamSynchronize(c->stream);
    return st;
}

extern "C" int pf_step(pf_ctx *c, int nsteps) {
    if (!c || !c->have_state) return pf_fail(PF_ERR_ARG, "pf_step: no state uploaded");
    if (nsteps < 0) return pf_fail(PF_ERR_ARG, "pf_step: negative step count");
    int s = 0;
    while (s < nsteps) {
        pf_step_params P;
        pf_compute_params(c->model, c->time, P);
        // Graph path: two steps with identical parameters return every buffer
        // to its role, so one captured pair is replayed.
        if (c->use_graph && !c->ktiming && s + 1 < nsteps) {
            pf_step_params P2;
            pf_compute_params(c->model, c->time + P.pfm_dt, P2);
            if (same_step(P, P2)) {
                const int sig = role_sig(c);
                if (!c->gexec || c->gphase != sig || !same_step(c->gparams, P)) {
                    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
                    cudaGraph_t g;
                    PF_CUDA_OK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                    cudaError_t e1 = launch_step(c, P);
                    cudaError_t e2 = launch_step(c, P2);
                    cudaError_t e3 = cudaStreamEndCapture(c->stream, &g);
                    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
                        return pf_cuda_fail(e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3));
                    cudaError_t e4 = cudaGraphInstantiate(&c->gexec, g, 0);
                    cudaGraphDestroy(g);
                    if (e4 != cudaSuccess) return pf_cuda_fail(e4);
                    c->gparams = P;
                    c->gphase = sig;  // roles are back where they started after two steps
                }
                PF_CUDA_OK(cudaGraphLaunch(c->gexec, c->stream));
                c->time += P.pfm_dt;
                c->time += P2.pfm_dt;
                c->last = P2;
                c->have_last = true;
                s += 2;
                continue;
            }
        }
        cudaError_t e = launch_step(c, P);
        if (e != cudaSuccess) return pf_cuda_fail(e);
        c->time += P.pfm_dt;  // phase_field.cpp:314
        c->last = P;
        c->have_last = true;
        s += 1;
    }
    return PF_OK;
}

extern "C" int pf_diffuse(pf_ctx *c, int nsub) {
    if (!c || !c->have_state) return pf_fail(PF_ERR_ARG, "pf_diffuse: no state uploaded");
    if (nsub < 0) return pf_fail(PF_ERR_ARG, "pf_diffuse: negative sub-step count");
    pf_step_params P;
    pf_compute_params(c->model, c->time, P);
    cudaError_t e = cudaSuccess;
    if (c->prec == PF_PREC_FP64) {
        if (nsub > 0) e = pf_launch_links_f64(P, P.nnb, c->phase, c->links, c->tpart, c->stream);
        for (int it = 0; it < nsub && e == cudaSuccess; it++) {
            const int b = c->curc;
            e = timed(c, 1, [&] {
                return pf_launch_diffuse_f64(P, P.nnb, P.coef_diff, c->links, c->tpart, c->conc[b], c->conc[1 - b],
                                             c->C, c->stream);
            });
            c->curc = 1 - b;
        }
    } else {
        pf_f32_params F;
        pf_fold_f32(P, c->map.off[2], c->map.off[3], F);
        for (int it = 0; it < nsub && e == cudaSuccess; it++) {
            const int b = c->curs;
            e = timed(c, 1, [&] { return pf_launch_diffuse_f32(F, c->phase32, c->sol[b], c->sol[1 - b], c->stream, c->diff_cfg_valid ? &c->diff_cfg : nullptr); });
            c->curs = 1 - b;
        }
    }
    return e == cudaSuccess ? PF_OK : pf_cuda_fail(e);
}

// Autotuner of the FP32 diffusion tile shape: every candidate (tile height x
// z chunk) runs on the context's own state, reading the current solute buffer
// and writing the spare one (which the next sub-step overwrites anyway), and
// the fastest mean of three timed launches is kept for this context.
extern "C" int pf_autotune(pf_ctx *c, int *ty, int *zchunk, int *variant, float *ms) {
    if (!c || !c->have_state) return pf_fail(PF_ERR_ARG, "pf_autotune: no state uploaded");
    if (c->prec != PF_PREC_FP32C) {
        if (ty) *ty = 0;
        if (zchunk) *zchunk = 0;
        if (variant) *variant = 0;
        if (ms) *ms = 0.f;
        return PF_OK;
    }
    pf_step_params P;
    pf_compute_params(c->model, c->time, P);
    pf_f32_params F;
    pf_fold_f32(P, c->map.off[2], c->map.off[3], F);
    pf_diff_cfg cand[32];
    const int nc = pf_diffuse_candidates(F, cand, 32);
    cudaEvent_t e0, e1;
    PF_CUDA_OK(cudaEventCreate(&e0));
    PF_CUDA_OK(cudaEventCreate(&e1));
    const int b = c->curs;
    float best = 1e30f;
    pf_diff_cfg best_cfg = pf_diffuse_default_cfg(F);
    int st = PF_OK;
    for (int i = 0; i < nc && st == PF_OK; i++) {
        cudaError_t e = pf_launch_diffuse_f32(F, c->phase32, c->sol[b], c->sol[1 - b], c->stream, &cand[i]);
        if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
        for (int r = 0; r < 3 && e == cudaSuccess; r++)
            e = pf_launch_diffuse_f32(F, c->phase32, c->sol[b], c->sol[1 - b], c->stream, &cand[i]);
        if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        if (e != cudaSuccess) st = pf_cuda_fail(e);
        else if (t / 3 < best) {
            best = t / 3;
            best_cfg = cand[i];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != PF_OK) return st;
    c->diff_cfg = best_cfg;
    c->diff_cfg_valid = true;
    c->diff_cfg_ms = best;
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; c->gphase = -1; }
    if (ty) *ty = best_cfg.ty;
    if (zchunk) *zchunk = best_cfg.zchunk;
    if (variant) *variant = best_cfg.variant;
    if (ms) *ms = best;
    return PF_OK;
}

extern "C" int pf_set_diffusion_tile(pf_ctx *c, int ty, int zchunk, int variant) {
    if (!c) return pf_fail(PF_ERR_ARG, "pf_set_diffusion_tile: null context");
    if (ty == 0) {  // back to the default rule
        c->diff_cfg_valid = false;
        return PF_OK;
    }
    pf_step_params P;
    pf_compute_params(c->model, c->time, P);
    pf_f32_params F;
    pf_fold_f32(P, c->map.off[2], c->map.off[3], F);
    if (zchunk < 1 || !pf_diffuse_variant_ok(F, ty, variant))
        return pf_fail(PF_ERR_ARG,
                       "pf_set_diffusion_tile: tile height 8/16/32 with variant 0, or 8/16 with variant 1 on a 3D grid "
                       "whose x extent is a multiple of 64 and y extent a multiple of the tile height; z chunk >= 1");
    c->diff_cfg = pf_diff_cfg{ty, zchunk, variant};
    c->diff_cfg_valid = true;
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; c->gphase = -1; }
    return PF_OK;
}

extern "C" int pf_diffusion_candidates(pf_ctx *c, int *out, int max) {
    if (!c || !out) return pf_fail(PF_ERR_ARG, "pf_diffusion_candidates: null argument");
    pf_step_params P;
    pf_compute_params(c->model, c->time, P);
    pf_f32_params F;
    pf_fold_f32(P, c->map.off[2], c->map.off[3], F);
    pf_diff_cfg cand[64];
    const int n = pf_diffuse_candidates(F, cand, 64);
    int k = 0;
    for (int i = 0; i < n && k < max; i++, k++) {
        out[3 * k] = cand[i].ty;
        out[3 * k + 1] = cand[i].zchunk;
        out[3 * k + 2] = cand[i].variant;
    }
    return k;
}

extern "C" int pf_reduce(pf_ctx *c, double out[8]) {
    if (!c || !c->have_state || !out) return pf_fail(PF_ERR_ARG, "pf_reduce: no state");
    cudaError_t e;
    if (c->prec == PF_PREC_FP64)
        e = pf_launch_reduce_f64(c->N, c->nsol, c->ids[c->cur], c->phi[c->cur], c->phase, c->C, c->partials,
                                 c->red_blocks, c->d_red, c->stream);
    else
        e = pf_launch_reduce_f32(c->N, c->nsol, c->map.off[1], c->gid[c->cur], c->phi32[c->cur], c->phase32,
                                 c->sol[c->curs], c->partials, c->red_blocks, c->d_red, c->stream);
    if (e != cudaSuccess) return pf_cuda_fail(e);
    PF_CUDA_OK(cudaMemcpyAsync(c->h_red, c->d_red, PF_RED_NOUT * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA_OK(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < PF_RED_NOUT; i++) out[i] = c->h_red[i];
    out[6] = 0.;
    if (c->nsol < 2) out[5] = 0.;
    return PF_OK;
}

extern "C" int pf_check_state(pf_ctx *c, const double reference_totals[2], double max_rel_drift, double out[8]) {
    double r[8];
    int st = pf_reduce(c, r);
    if (st != PF_OK) return st;
    if (out)
        for (int i = 0; i < 8; i++) out[i] = r[i];
    if (r[7] > 0) return pf_fail(PF_ERR_NONFINITE, "pf_check_state: non-finite values in the state");
    if (reference_totals && max_rel_drift > 0)
        for (int q = 0; q < c->nsol; q++) {
            const double ref = reference_totals[q];
            if (ref != 0.0 && std::abs(r[4 + q] - ref) > max_rel_drift * std::abs(ref))
                return pf_fail(PF_ERR_DRIFT, "pf_check_state: solute total drifted beyond the tolerance");
        }
    return PF_OK;
}

extern "C" int pf_synchronize(pf_ctx *c) {
    if (!c) return pf_fail(PF_ERR_ARG, "pf_synchronize: null context");
    PF_CUDA_OK(cudaStreamSynchronize(c->stream));
    if (pf_diffuse_take_timeout())
        return pf_fail(PF_ERR_TIMEOUT, "pf_synchronize: a bounded wait of the staged diffusion kernel ran out");
    if (c->model.drag && pf_drag_take_failure())
        return pf_fail(PF_ERR_RANGE, "pf_synchronize: a solute-drag velocity iteration found no root "
                                     "(the Fortran model stops there)");
    return PF_OK;
}

extern "C" int pf_get_time(pf_ctx *c, double *t) {
    if (!c || !t) return pf_fail(PF_ERR_ARG, "pf_get_time: null argument");
    *t = c->time;
    return PF_OK;
}

extern "C" int pf_last_params(pf_ctx *c, pf_step_params *out) {
    if (!c || !out) return pf_fail(PF_ERR_ARG, "pf_last_params: null argument");
    if (c->have_last) *out = c->last;
    else pf_compute_params(c->model, c->time, *out);
    return PF_OK;
}

extern "C" int pf_truncated_cells(pf_ctx *c, long long *out) {
    if (!c || !out) return pf_fail(PF_ERR_ARG, "pf_truncated_cells: null argument");
    *out = c->truncated;
    return PF_OK;
}

extern "C" int pf_enable_kernel_timing(pf_ctx *c, int on) {
    if (!c) return pf_fail(PF_ERR_ARG, "pf_enable_kernel_timing: null context");
    int st = collect_times(c);
    c->ktiming = on != 0;
    c->ktime[0] = c->ktime[1] = 0.;
    c->kcount[0] = c->kcount[1] = 0;
    return st;
}

extern "C" int pf_kernel_times(pf_ctx *c, double times_ms[2], long long counts[2]) {
    if (!c || !times_ms || !counts) return pf_fail(PF_ERR_ARG, "pf_kernel_times: null argument");
    int st = collect_times(c);
    for (int i = 0; i < 2; i++) {
        times_ms[i] = c->ktime[i];
        counts[i] = c->kcount[i];
    }
    return st;
}

extern "C" int pf_use_graph(pf_ctx *c, int on) {
    if (!c) return pf_fail(PF_ERR_ARG, "pf_use_graph: null context");
    c->use_graph = on != 0;
    return PF_OK;
}

// ===========================================================================
// 3. Batched 2D domains: one persistent cooperative launch (pf_batch.cu).
// ===========================================================================
struct pf_batch {
    std::vector<pf_ctx *> dom;
    int nsol = 1;
    cudaStream_t stream = nullptr;
    pf_batch_dom *h_doms = nullptr, *d_doms = nullptr;
    pf_f32_params *h_params = nullptr, *d_params = nullptr;
    int *h_block_dom = nullptr, *d_block_dom = nullptr;
    int max_blocks = 0, nblocks = 0;
    unsigned long long *d_ctr = nullptr;
    int *d_err = nullptr, *h_err = nullptr;
    unsigned long long timeout_ns = 2000000000ull;  // 2 s per barrier wait
    int extra_target = 0;
    cudaGraphExec_t gexec = nullptr;
    int g_steps = -1, g_blocks = -1, g_tile = -1;
    // Tile height of the persistent kernel and the fraction (1/occ_div) of
    // the resident-block capacity it uses: chosen by pf_batch_autotune.
    int tile_y = 8, occ_div = 1;
    int sms = 0;
};

namespace {
void batch_free(pf_batch *b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (auto c : b->dom) pf_destroy(c);
    cudaFree(b->d_doms); cudaFree(b->d_params); cudaFree(b->d_block_dom); cudaFree(b->d_ctr); cudaFree(b->d_err);
    cudaFreeHost(b->h_doms); cudaFreeHost(b->h_params); cudaFreeHost(b->h_block_dom); cudaFreeHost(b->h_err);
    if (b->stream) cudaStreamDestroy(b->stream);
}
}  // namespace

extern "C" int pf_batch_create(const pf_model *models, int ndom, pf_batch **out) {
    if (!models || !out || ndom < 1) return pf_fail(PF_ERR_ARG, "pf_batch_create: bad arguments");
    *out = nullptr;
    for (int d = 0; d < ndom; d++) {
        const pf_model &m = models[d];
        if (m.iz != 1) return pf_fail(PF_ERR_ARG, "pf_batch_create: batched domains are 2D (iz == 1)");
        if (m.nsol != models[0].nsol) return pf_fail(PF_ERR_ARG, "pf_batch_create: all domains need the same solutes");
        if (m.avg_carbon || m.drag || m.coherent)
            return pf_fail(PF_ERR_ARG,
                           "pf_batch_create: the interface-averaged carbon, the solute drag and the coherent-grain "
                           "mobility run on the FP64 path only");
        for (int t = 1; t < m.nT; t++)
            if (m.T_temp[t] != m.T_temp[0])
                return pf_fail(PF_ERR_ARG, "pf_batch_create: each domain needs a constant temperature");
    }
    pf_batch *b = new pf_batch();
    b->nsol = models[0].nsol;
    int st = PF_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) st = pf_cuda_fail(e);
    for (int d = 0; d < ndom && st == PF_OK; d++) {
        pf_ctx *c = nullptr;
        st = pf_create(&models[d], PF_PREC_FP32C, &c);
        if (st == PF_OK) {
            b->dom.push_back(c);
            st = pf_set_stream(c, b->stream);
        }
    }
    int dev = 0, sms = 0;
    if (st == PF_OK) {
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        b->sms = sms;
        // Capacity for the largest candidate launch (4-row tiles, full occupancy).
        b->max_blocks = pf_batch_blocks_per_sm(b->nsol, 4) * sms;
        if (pf_batch_blocks_per_sm(b->nsol, 8) * sms < ndom)
            st = pf_fail(PF_ERR_RANGE, "pf_batch_create: more domains than resident blocks");
    }
    bool ok = st == PF_OK;
    auto dalloc = [&](void **p, size_t n) { if (ok && cudaMalloc(p, n) != cudaSuccess) ok = false; };
    auto halloc = [&](void **p, size_t n) { if (ok && cudaMallocHost(p, n) != cudaSuccess) ok = false; };
    dalloc((void **)&b->d_doms, sizeof(pf_batch_dom) * ndom);
    dalloc((void **)&b->d_params, sizeof(pf_f32_params) * ndom);
    dalloc((void **)&b->d_block_dom, sizeof(int) * (b->max_blocks > 0 ? b->max_blocks : 1));
    dalloc((void **)&b->d_ctr, sizeof(unsigned long long) * ndom);
    dalloc((void **)&b->d_err, sizeof(int));
    halloc((void **)&b->h_doms, sizeof(pf_batch_dom) * ndom);
    halloc((void **)&b->h_params, sizeof(pf_f32_params) * ndom);
    halloc((void **)&b->h_block_dom, sizeof(int) * (b->max_blocks > 0 ? b->max_blocks : 1));
    halloc((void **)&b->h_err, sizeof(int));
    if (st == PF_OK && !ok) {
        cudaGetLastError();
        st = pf_fail(PF_ERR_NOMEM, "pf_batch_create: allocation failed");
    }
    if (st != PF_OK) {
        batch_free(b);
        delete b;
        return st;
    }
    *out = b;
    return PF_OK;
}

extern "C" int pf_batch_destroy(pf_batch *b) {
    if (!b) return PF_OK;
    cudaStreamSynchronize(b->stream);
    batch_free(b);
    delete b;
    return PF_OK;
}

static int batch_dom_check(pf_batch *b, int d) {
    if (!b || d < 0 || d >= (int)b->dom.size()) return pf_fail(PF_ERR_ARG, "pf_batch: bad domain index");
    return PF_OK;
}

extern "C" int pf_batch_upload(pf_batch *b, int d, const int32_t *ids, const double *phi, const double *phase,
                               const double *C, double time) {
    int st = batch_dom_check(b, d);
    if (st != PF_OK) return st;
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
    return pf_upload_state(b->dom[d], ids, phi, phase, nullptr, C, time);
}

extern "C" int pf_batch_download(pf_batch *b, int d, int32_t *ids, double *phi, double *phase, double *conc,
                                 double *C, double *time) {
    int st = batch_dom_check(b, d);
    if (st != PF_OK) return st;
    return pf_download_state(b->dom[d], ids, phi, phase, conc, C, time);
}

extern "C" int pf_batch_reduce(pf_batch *b, int d, double out[8]) {
    int st = batch_dom_check(b, d);
    if (st != PF_OK) return st;
    return pf_reduce(b->dom[d], out);
}

extern "C" int pf_batch_set_timeout(pf_batch *b, unsigned long long timeout_ns, int unreachable_barrier) {
    if (!b) return pf_fail(PF_ERR_ARG, "pf_batch_set_timeout: null batch");
    b->timeout_ns = timeout_ns;
    b->extra_target = unreachable_barrier ? 1 : 0;
    return PF_OK;
}

extern "C" int pf_batch_info(pf_batch *b, long long out[4]) {
    if (!b || !out) return pf_fail(PF_ERR_ARG, "pf_batch_info: null argument");
    long long cells = 0;
    int nsub_max = 0;
    for (auto c : b->dom) {
        cells += c->N;
        pf_step_params P;
        pf_compute_params(c->model, c->time, P);
        if (P.n_sub > nsub_max) nsub_max = P.n_sub;
    }
    out[0] = cells;
    out[1] = b->nblocks > 0 ? b->nblocks : b->max_blocks;
    out[2] = (long long)b->dom.size();
    out[3] = nsub_max;
    return PF_OK;
}

extern "C" int pf_batch_run(pf_batch *b, int nsteps) {
    if (!b || nsteps < 0) return pf_fail(PF_ERR_ARG, "pf_batch_run: bad arguments");
    const int nd = (int)b->dom.size();
    for (auto c : b->dom)
        if (!c->have_state) return pf_fail(PF_ERR_ARG, "pf_batch_run: a domain has no state");
    if (nsteps == 0) return PF_OK;
    // Parameters, and block groups sized by work (phase sweep ~ 2 sub-steps).
    const int ty_tile = b->tile_y;
    const int cap = pf_batch_blocks_per_sm(b->nsol, ty_tile) * b->sms / b->occ_div;
    if (cap < nd) return pf_fail(PF_ERR_RANGE, "pf_batch_run: more domains than resident blocks for this tile shape");
    std::vector<double> w(nd);
    std::vector<int> tiles(nd), nsub(nd);
    double wsum = 0.;
    for (int d = 0; d < nd; d++) {
        pf_ctx *c = b->dom[d];
        pf_step_params P;
        pf_compute_params(c->model, c->time, P);
        pf_fold_f32(P, c->map.off[2], c->map.off[3], b->h_params[d]);
        nsub[d] = P.n_sub;
        const int tx = (c->model.ix + 31) / 32, ty = (c->model.iy + ty_tile - 1) / ty_tile;
        tiles[d] = tx * ty;
        w[d] = (double)c->N * (2 + P.n_sub);
        wsum += w[d];
        b->h_doms[d].tiles_x = tx;
        b->h_doms[d].tiles = tiles[d];
    }
    std::vector<int> nb(nd);
    int used = 0;
    for (int d = 0; d < nd; d++) {
        nb[d] = (int)((double)cap * w[d] / wsum);
        if (nb[d] < 1) nb[d] = 1;
        if (nb[d] > tiles[d]) nb[d] = tiles[d];
        used += nb[d];
    }
    while (used > cap) {  // trim the largest groups
        int big = 0;
        for (int d = 1; d < nd; d++)
            if (nb[d] > nb[big]) big = d;
        nb[big]--;
        used--;
    }
    int first = 0;
    for (int d = 0; d < nd; d++) {
        pf_ctx *c = b->dom[d];
        pf_batch_dom &D = b->h_doms[d];
        D.gid[0] = c->gid[0]; D.gid[1] = c->gid[1];
        D.phi[0] = c->phi32[0]; D.phi[1] = c->phi32[1];
        D.sph = c->phase32;
        D.sol[0] = c->sol[0]; D.sol[1] = c->sol[1];
        D.cur = c->cur; D.curs = c->curs;
        D.nb_first = first;
        D.nb = nb[d];
        D.extra_target = b->extra_target;
        for (int k = 0; k < nb[d]; k++) b->h_block_dom[first + k] = d;
        first += nb[d];
    }
    b->nblocks = used;
    // One graph per (steps, block count): the memcpy nodes read the pinned
    // host tables at replay, so updated buffer roles and parameters flow in.
    if (!b->gexec || b->g_steps != nsteps || b->g_blocks != used || b->g_tile != ty_tile) {
        if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
        cudaGraph_t g;
        PF_CUDA_OK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaMemcpyAsync(b->d_doms, b->h_doms, sizeof(pf_batch_dom) * nd, cudaMemcpyHostToDevice, b->stream);
        cudaMemcpyAsync(b->d_params, b->h_params, sizeof(pf_f32_params) * nd, cudaMemcpyHostToDevice, b->stream);
        cudaMemcpyAsync(b->d_block_dom, b->h_block_dom, sizeof(int) * used, cudaMemcpyHostToDevice, b->stream);
        cudaMemsetAsync(b->d_ctr, 0, sizeof(unsigned long long) * nd, b->stream);
        cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream);
        cudaError_t e1 = pf_launch_batch(b->nsol, ty_tile, used, b->d_doms, b->d_params, b->d_block_dom, nsteps,
                                         b->d_ctr, b->d_err, b->timeout_ns, b->stream);
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        if (e1 != cudaSuccess || e2 != cudaSuccess) return pf_cuda_fail(e1 != cudaSuccess ? e1 : e2);
        cudaError_t e3 = cudaGraphInstantiate(&b->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e3 != cudaSuccess) return pf_cuda_fail(e3);
        b->g_steps = nsteps;
        b->g_blocks = used;
        b->g_tile = ty_tile;
    }
    PF_CUDA_OK(cudaGraphLaunch(b->gexec, b->stream));
    PF_CUDA_OK(cudaMemcpyAsync(b->h_err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    PF_CUDA_OK(cudaStreamSynchronize(b->stream));
    if (*b->h_err) return pf_fail(PF_ERR_TIMEOUT, "pf_batch_run: a domain barrier timed out; the launch was abandoned");
    for (int d = 0; d < nd; d++) {
        pf_ctx *c = b->dom[d];
        c->cur ^= (nsteps & 1);
        c->curs ^= ((long long)nsteps * nsub[d]) & 1;
        pf_step_params P;
        for (int s = 0; s < nsteps; s++) {  // the same time accumulation as pf_step
            pf_compute_params(c->model, c->time, P);
            c->time += P.pfm_dt;
        }
        c->last = P;
        c->have_last = true;
    }
    return PF_OK;
}

extern "C" int pf_batch_set_tile(pf_batch *b, int tile_y, int occupancy_divisor) {
    if (!b || !pf_batch_tile_ok(tile_y) || occupancy_divisor < 1 || occupancy_divisor > 4)
        return pf_fail(PF_ERR_ARG, "pf_batch_set_tile: tile height 4 or 8, occupancy divisor 1..4");
    b->tile_y = tile_y;
    b->occ_div = occupancy_divisor;
    return PF_OK;
}

// Autotuner of the persistent kernel's shape: each candidate (tile height x
// fraction of the resident-block capacity) advances every domain nsteps from
// the current states -- once to build its graph, once timed -- and the states
// are restored after every trial, so the ensemble is left exactly as it was.
extern "C" int pf_batch_autotune(pf_batch *b, int nsteps, int *tile_y, int *occupancy_divisor, float *ms) {
    if (!b || nsteps < 1) return pf_fail(PF_ERR_ARG, "pf_batch_autotune: bad arguments");
    struct Snap {
        void *buf[7];
        size_t bytes[7];
        int cur, curs;
        double time;
        pf_step_params last;
        bool have_last;
    };
    std::vector<Snap> snap(b->dom.size());
    int st = PF_OK;
    for (size_t d = 0; d < b->dom.size() && st == PF_OK; d++) {
        pf_ctx *c = b->dom[d];
        if (!c->have_state) return pf_fail(PF_ERR_ARG, "pf_batch_autotune: a domain has no state");
        const size_t N = (size_t)c->N;
        void *src[7] = {c->gid[0], c->gid[1], c->phi32[0], c->phi32[1], c->phase32, c->sol[0], c->sol[1]};
        const size_t by[7] = {N * sizeof(ushort4), N * sizeof(ushort4), N * sizeof(float4), N * sizeof(float4),
                              3 * N * sizeof(float), N * c->nsol * sizeof(float2), N * c->nsol * sizeof(float2)};
        Snap &S = snap[d];
        for (int k = 0; k < 7; k++) {
            S.buf[k] = nullptr;
            S.bytes[k] = by[k];
            if (st == PF_OK && cudaMalloc(&S.buf[k], by[k]) != cudaSuccess) {
                cudaGetLastError();
                st = pf_fail(PF_ERR_NOMEM, "pf_batch_autotune: snapshot allocation failed");
            }
            if (st == PF_OK) cudaMemcpyAsync(S.buf[k], src[k], by[k], cudaMemcpyDeviceToDevice, b->stream);
        }
        S.cur = c->cur; S.curs = c->curs; S.time = c->time; S.last = c->last; S.have_last = c->have_last;
    }
    auto restore = [&]() {
        for (size_t d = 0; d < b->dom.size(); d++) {
            pf_ctx *c = b->dom[d];
            void *dst[7] = {c->gid[0], c->gid[1], c->phi32[0], c->phi32[1], c->phase32, c->sol[0], c->sol[1]};
            const Snap &S = snap[d];
            for (int k = 0; k < 7; k++) cudaMemcpyAsync(dst[k], S.buf[k], S.bytes[k], cudaMemcpyDeviceToDevice, b->stream);
            c->cur = S.cur; c->curs = S.curs; c->time = S.time; c->last = S.last; c->have_last = S.have_last;
        }
    };
    const int old_ty = b->tile_y, old_div = b->occ_div;
    int best_ty = old_ty, best_div = old_div;
    float best = 1e30f;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (st == PF_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
        st = pf_fail(PF_ERR_CUDA, "pf_batch_autotune: event creation failed");
    const int tys[2] = {4, 8}, divs[2] = {1, 2};
    for (int a = 0; a < 2 && st == PF_OK; a++)
        for (int v = 0; v < 2 && st == PF_OK; v++) {
            b->tile_y = tys[a];
            b->occ_div = divs[v];
            if (pf_batch_blocks_per_sm(b->nsol, tys[a]) * b->sms / divs[v] < (int)b->dom.size()) continue;
            restore();
            st = pf_batch_run(b, nsteps);  // builds this shape's graph
            if (st != PF_OK) break;
            restore();
            cudaEventRecord(e0, b->stream);
            st = pf_batch_run(b, nsteps);
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (st == PF_OK && t < best) {
                best = t;
                best_ty = tys[a];
                best_div = divs[v];
            }
        }
    if (!snap.empty() && snap[0].buf[0]) restore();
    cudaStreamSynchronize(b->stream);
    for (auto &S : snap)
        for (int k = 0; k < 7; k++) cudaFree(S.buf[k]);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st != PF_OK) {
        b->tile_y = old_ty;
        b->occ_div = old_div;
        return st;
    }
    b->tile_y = best_ty;
    b->occ_div = best_div;
    if (tile_y) *tile_y = best_ty;
    if (occupancy_divisor) *occupancy_divisor = best_div;
    if (ms) *ms = best;
    return PF_OK;
}

extern "C" int pf_write_data(pf_ctx *c, const char *directory, int forced, int *written) {
    if (!c || !directory) return pf_fail(PF_ERR_ARG, "pf_write_data: null argument");
    if (written) *written = 0;
    pf_step_params P;
    pf_last_params(c, &P);
    const double temperature = P.T;
    if (!(forced || pf_output_due(c->time, c->model.timestep_output, P.pfm_dt, temperature,
                                  c->last_temperature_written)))
        return PF_OK;
    double r[8];
    int st = pf_reduce(c, r);
    if (st != PF_OK) return st;
    const double vol = (double)c->model.ix * c->model.iy * c->model.iz;
    double fr[3] = {r[0] / vol, r[1] / vol, r[2] / vol};
    std::string line = pf_format_fraction_line(c->time, temperature, fr, r[3] / vol);
    std::ofstream k(std::string(directory) + "/fraction_time.txt", std::ios::app);
    if (!k.is_open()) return pf_fail(PF_ERR_IO, "pf_write_data: cannot open fraction_time.txt");
    k << line;
    if (c->model.micro_out) {
        const size_t N = (size_t)c->N;
        std::vector<int32_t> ids(6 * N);
        std::vector<double> C(N * c->nsol);
        st = pf_download_state(c, ids.data(), nullptr, nullptr, nullptr, C.data(), nullptr);
        if (st != PF_OK) return st;
        char name[64];
        std::snprintf(name, sizeof(name), "field%07d_%d.vti", (int)(c->time * 100), c->micro_count);
        st = pf_write_vti((std::string(directory) + "/" + name).c_str(), c->model.ix, c->model.iy, c->model.iz,
                          c->model.dx, ids.data(), C.data());
        if (st != PF_OK) return st;
        c->micro_count++;
    }
    c->last_temperature_written = temperature;
    if (written) *written = 1;
    return PF_OK;
}

// ===========================================================================
// 4. Binary microstructure files from device buffers (pf_output.cu).
// ===========================================================================
extern "C" int pf_write_vti_binary(pf_ctx *c, const char *directory, int index, int pieces) {
    if (!c || !directory || index < 0 || pieces < 1) return pf_fail(PF_ERR_ARG, "pf_write_vti_binary: bad argument");
    if (!c->have_state) return pf_fail(PF_ERR_ARG, "pf_write_vti_binary: no state uploaded");
    if (!c->out) c->out = pf_out_create();
    const pf_model &m = c->model;
    if (c->prec == PF_PREC_FP64)
        return pf_out_write_fp64(c->out, c->stream, m.ix, m.iy, m.iz, m.dx, c->ids[c->cur], c->C, directory, index,
                                 pieces);
    return pf_out_write_fp32(c->out, c->stream, m.ix, m.iy, m.iz, m.dx, c->nsol, c->map.off[2], c->map.off[3],
                             c->gid[c->cur], c->sol[c->curs], directory, index, pieces);
}

extern "C" int pf_write_wait(pf_ctx *c) {
    if (!c) return pf_fail(PF_ERR_ARG, "pf_write_wait: null context");
    return pf_out_wait(c->out);
}

// ===========================================================================
// 5. Seeded initial state generated on the device (pf_init_dev.cu).
// ===========================================================================
extern "C" int pf_init_device(pf_ctx *c, const pf_init_spec *spec, double time) {
    if (!c || !spec) return pf_fail(PF_ERR_ARG, "pf_init_device: null argument");
    const pf_model &m = c->model;
    pf_step_params P;
    pf_compute_params(m, time, P);
    c->time = time;
    c->cur = c->curc = c->curs = 0;
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; c->gphase = -1; }
    const char *msg = nullptr;
    int st;
    if (c->prec == PF_PREC_FP64) {
        st = pf_init_generate_device(m.ix, m.iy, m.iz, c->nsol, m.cutoff, spec, &P.k[0][0], &P.c[0][0], c->ids[0],
                                     c->phi[0], c->phase, c->conc[0], c->C, c->stream, &msg);
    } else {
        if (!ensure_staging(c, false)) return pf_fail(PF_ERR_NOMEM, "pf_init_device: staging allocation failed");
        st = pf_init_generate_device(m.ix, m.iy, m.iz, c->nsol, m.cutoff, spec, nullptr, nullptr, c->st_ids,
                                     c->st_phi, c->st_phase, nullptr, c->st_C, c->stream, &msg);
        if (st == PF_OK) {
            c->have_state = false;
            st = pack_staged(c, "pf_init_device");
            if (st != PF_OK) return st;
        }
    }
    if (st != PF_OK) return pf_fail(st, std::string("pf_init_device: ") + (msg ? msg : "failed"));
    c->have_state = true;
    c->have_last = false;
    return PF_OK;
}
