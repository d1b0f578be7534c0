// arap_server.cpp -- arap_srv_* (include/arap_gpu.h): the scheduler of
// arap_server.h over the library's device contexts.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <string>

#include "../../include/arap_gpu.h"
#include "arap_server.h"

namespace {

// Backend of the scheduler: the library's contexts, pinned host staging.
struct CtxBackend {
    using Handle = arap_ctx *;
    static constexpr bool kCallbacks = true;
    int device = 0;

    int create(int V, int F, const int32_t *faces, Handle *h) { return arap_create(V, F, faces, device, h); }
    int create_like(Handle src, Handle *h) { return arap_create_like(src, h); }
    void destroy(Handle h) { arap_destroy(h); }
    int set_precision(Handle h, int prec, int refine) { return arap_set_precision(h, prec, refine); }
    int set_rest(Handle h, const double *xyz) { return arap_set_rest_positions(h, xyz); }
    int set_solve_ctas(Handle h, int n) { return arap_set_solve_ctas(h, n); }
    int set_ordering(Handle h, int mode) { return arap_set_ordering(h, mode); }
    int set_constraints(Handle h, int n, const int32_t *idx, const double *xyz) {
        return arap_set_constraints(h, n, idx, xyz);
    }
    int set_targets(Handle h, int n, const double *xyz) { return arap_set_targets(h, n, xyz); }
    int plan_bytes(Handle h, int P, int64_t *bytes) { return arap_plan_bytes(h, P, bytes); }
    int64_t device_bytes(Handle h) { return arap_device_bytes(h); }
    int deform_async(Handle h, int iters, double *out) { return arap_deform_async(h, iters, out); }
    int deform_poses_async(Handle h, int P, const double *tgt, int iters, double *out) {
        return arap_deform_poses_async(h, P, tgt, iters, out);
    }
    int query(Handle h, int32_t *done) { return arap_query(h, done); }
    int set_done_callback(Handle h, void (*fn)(void *), void *user) { return arap_set_done_callback(h, fn, user); }
    void host_timing(Handle h, double *ms5) {
        if (arap_get_host_timing(h, ms5) != ARAP_OK)
            for (int i = 0; i < 5; ++i) ms5[i] = 0.0;
    }
    double device_ms(Handle h) {
        double a = 0.0, b = 0.0;
        return arap_get_timing(h, &a, &b) == ARAP_OK ? a + b : 0.0;
    }
    std::string last_error(Handle h) { return arap_last_error(h); }
    void *alloc_host(size_t bytes) {
        void *p = nullptr;
        return cudaMallocHost(&p, bytes) == cudaSuccess ? p : nullptr;
    }
    void free_host(void *p) { cudaFreeHost(p); }
    // Grows the device's stream-ordered pool by `bytes` once (allocated and
    // freed again; freed pool memory stays with the process): the contexts of
    // new constraint sets then take their buffers from memory the process
    // already holds instead of mapping more from the driver (measured ~6.7 ms
    // of buffer allocation per new set on a growing pool).
    void reserve_pool(int64_t bytes) {
        if (bytes <= 0) return;
        cudaSetDevice(device);
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) != cudaSuccess) return;
        uint64_t thr = ~0ull;
        if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr) != cudaSuccess) return;
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return;
        void *p = nullptr;
        if (cudaMallocAsync(&p, (size_t)bytes, st) == cudaSuccess) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
        cudaGetLastError();  // a reservation that did not fit is not an error of the server
    }
    int64_t default_budget() {
        size_t free_b = 0, total_b = 0;
        cudaSetDevice(device);
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
        return (int64_t)(0.8 * (double)free_b);
    }
};

}  // namespace

struct arap_server {
    arapsrv::Server<CtxBackend> *impl = nullptr;
};

extern "C" {

int arap_srv_create(const arap_server_config *cfg, arap_server **out) {
    arapsrv::thread_error().clear();
    if (!cfg || !out) {
        arapsrv::thread_error() = "arap_srv_create: invalid argument";
        return ARAP_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        arapsrv::thread_error() = "no CUDA device visible";
        return ARAP_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev || cfg->refine_steps < 0 || cfg->refine_steps > 8 ||
        (cfg->precision != ARAP_PRECISION_FP64 && cfg->precision != ARAP_PRECISION_MIXED)) {
        arapsrv::thread_error() = "arap_srv_create: device, precision or refine_steps out of range";
        return ARAP_ERR_INVALID_ARGUMENT;
    }
    CtxBackend b;
    b.device = cfg->device;
    {
        // pool memory for the contexts to come: a quarter of the budget, at
        // most 32 GiB
        const int64_t budget = cfg->device_budget_bytes > 0 ? cfg->device_budget_bytes : b.default_budget();
        b.reserve_pool(std::min<int64_t>(budget / 4, (int64_t)32 << 30));
    }
    arap_server *s = new (std::nothrow) arap_server();
    if (!s) return ARAP_ERR_OUT_OF_MEMORY;
    s->impl = new arapsrv::Server<CtxBackend>(b, *cfg);
    *out = s;
    return ARAP_OK;
}

void arap_srv_destroy(arap_server *srv) {
    if (!srv) return;
    delete srv->impl;
    delete srv;
}

int arap_srv_add_mesh(arap_server *srv, int32_t n_vertices, int32_t n_faces, const int32_t *faces,
                      const double *rest_xyz, int32_t *mesh_id) {
    if (!srv) return ARAP_ERR_INVALID_ARGUMENT;
    return srv->impl->add_mesh(n_vertices, n_faces, faces, rest_xyz, mesh_id);
}

int arap_srv_submit(arap_server *srv, const arap_request *req, int64_t *ticket) {
    if (!srv) return ARAP_ERR_INVALID_ARGUMENT;
    return srv->impl->submit(req, ticket);
}

int arap_srv_poll(arap_server *srv, int64_t ticket, arap_request_info *info) {
    if (!srv) return ARAP_ERR_INVALID_ARGUMENT;
    return srv->impl->poll(ticket, info);
}

int arap_srv_wait(arap_server *srv, int64_t ticket, int32_t timeout_ms, arap_request_info *info) {
    if (!srv) return ARAP_ERR_INVALID_ARGUMENT;
    return srv->impl->wait(ticket, timeout_ms, info);
}

int arap_srv_stats(arap_server *srv, arap_server_stats *stats) {
    if (!srv || !stats) return ARAP_ERR_INVALID_ARGUMENT;
    srv->impl->stats(stats);
    return ARAP_OK;
}

const char *arap_srv_last_error(const arap_server *) { return arapsrv::thread_error().c_str(); }

}  // extern "C"
