// arap_noalloc.cu -- cotan edge weights without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need the
// weights: a per-frame callback of an interactive viewer (the reference's
// examples deform inside one, examples/osg_viewer.cpp:45-72) must not stall on
// cudaMalloc, which synchronises the device, and a host application that owns
// every byte of device memory through its own pool forbids driver allocations
// altogether. For them arap_cotan_weights_static computes _edgeWeights
// (inc/deform/arap.h:182-239) into buffers the caller already owns, keeping its
// one scratch array -- the three cotangent halves of every face -- in a
// file-scope __device__ array instead of memory obtained with cudaMalloc.
//
// Limits and sharing: the array holds kStaticMaxFaces faces (12 MiB) and exists
// on every device that loads the library until the process exits. All calls on
// a device share it and it keeps the last call's contents; calls whose kernels
// overlap on the GPU (different streams, or different host threads on the same
// device) race on it and must be ordered by the caller.
//
// Input checks on the device: the face indices and the weight pattern live in
// device memory, so they are checked by the kernels, not the host. A face with
// an index outside [0, n_vertices) is skipped (its scratch halves are zero and
// nothing is added for it), and an edge whose entry is missing from the
// pattern adds nothing; every such event is counted in a file-scope __device__
// counter that arap_cotan_weights_static_status reads. No kernel reads outside
// faces[0, 3F), xyz[0, 3V), rowptr[0, V] or col/val[0, nnz).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/arap_gpu.h"

namespace arapgpu {
void set_global_error(const std::string &msg);
}

namespace {

constexpr int kStaticMaxFaces = 1 << 19;  // 524,288 faces
constexpr int kMaxDevices = 64;

// per-face cotangent halves (arap.h:212-227), three doubles per face
static __device__ __align__(256) double g_face_cot_scratch[3 * kStaticMaxFaces];
// faces skipped for an out-of-range index plus edges missing from the pattern,
// in the last call on this device (zeroed at the start of every call)
static __device__ int g_skipped;

std::mutex g_setup_mutex;
double *g_scratch_addr[kMaxDevices] = {};
int *g_skipped_addr[kMaxDevices] = {};

// Host code cannot use g_face_cot_scratch or g_skipped as device addresses (in
// host code their names denote host-side stand-ins). Their device addresses
// are looked up once per device, with that device current, and passed to the
// kernels and copies.
cudaError_t symbol_addresses(int device, double **scratch, int **skipped) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void *p = nullptr, *q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_face_cot_scratch);
        if (e != cudaSuccess) return e;
        e = cudaGetSymbolAddress(&q, g_skipped);
        if (e != cudaSuccess) return e;
        g_skipped_addr[device] = static_cast<int *>(q);
        g_scratch_addr[device] = static_cast<double *>(p);
    }
    *scratch = g_scratch_addr[device];
    *skipped = g_skipped_addr[device];
    return cudaSuccess;
}

int current_device(int *device) {
    if (cudaGetDevice(device) != cudaSuccess || *device < 0 || *device >= kMaxDevices) return ARAP_ERR_NO_DEVICE;
    return ARAP_OK;
}

__device__ __forceinline__ bool in_range(int v, int n) { return v >= 0 && v < n; }

// The clamped Heron cotangents of arap.h:199-218 times 1/2, each operation
// rounded separately (no fused multiply-add), as the FP64 CPU path does. A
// face with an index outside [0, V) reads no position, gets zero halves and is
// counted.
__global__ void k_face_cots_to_scratch(int F, int V, const int32_t *__restrict__ faces,
                                       const double *__restrict__ xyz, double *__restrict__ hc, int *skipped) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    const int i0 = faces[3 * f], i1 = faces[3 * f + 1], i2 = faces[3 * f + 2];
    if (!in_range(i0, V) || !in_range(i1, V) || !in_range(i2, V)) {
        hc[3 * (int64_t)f + 0] = 0.0;
        hc[3 * (int64_t)f + 1] = 0.0;
        hc[3 * (int64_t)f + 2] = 0.0;
        atomicAdd(skipped, 1);
        return;
    }
    const double *v0 = xyz + 3 * (int64_t)i0, *v1 = xyz + 3 * (int64_t)i1, *v2 = xyz + 3 * (int64_t)i2;
    double l0 = 0.0, l1 = 0.0, l2 = 0.0, d;
    for (int c = 0; c < 3; ++c) { d = __dsub_rn(v1[c], v0[c]); l0 = __dadd_rn(l0, __dmul_rn(d, d)); }
    for (int c = 0; c < 3; ++c) { d = __dsub_rn(v2[c], v1[c]); l1 = __dadd_rn(l1, __dmul_rn(d, d)); }
    for (int c = 0; c < 3; ++c) { d = __dsub_rn(v0[c], v2[c]); l2 = __dadd_rn(l2, __dmul_rn(d, d)); }
    l0 = __dsqrt_rn((1e-8 < l0) ? l0 : 1e-8);
    l1 = __dsqrt_rn((1e-8 < l1) ? l1 : 1e-8);
    l2 = __dsqrt_rn((1e-8 < l2) ? l2 : 1e-8);
    const double s = __dmul_rn(0.5, __dadd_rn(__dadd_rn(l0, l1), l2));
    double area = __dsqrt_rn(
        __dmul_rn(__dmul_rn(__dmul_rn(s, __dsub_rn(s, l0)), __dsub_rn(s, l1)), __dsub_rn(s, l2)));
    area = (1e-8 < area) ? area : 1e-8;
    const double denom = __ddiv_rn(1.0, __dmul_rn(4.0, area));
    const double q0 = __dmul_rn(l0, l0), q1 = __dmul_rn(l1, l1), q2 = __dmul_rn(l2, l2);
    double c0 = __dmul_rn(__dadd_rn(__dadd_rn(-q0, q1), q2), denom);
    double c1 = __dmul_rn(__dadd_rn(__dsub_rn(q0, q1), q2), denom);
    double c2 = __dmul_rn(__dsub_rn(__dadd_rn(q0, q1), q2), denom);
    hc[3 * (int64_t)f + 0] = __dmul_rn((1e-10 < c0) ? c0 : 1e-10, 0.5);
    hc[3 * (int64_t)f + 1] = __dmul_rn((1e-10 < c1) ? c1 : 1e-10, 0.5);
    hc[3 * (int64_t)f + 2] = __dmul_rn((1e-10 < c2) ? c2 : 1e-10, 0.5);
}

// val = 0; thread 0 also clears the skip counter of the previous call
__global__ void k_zero(int n, double *__restrict__ v, int *skipped) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *skipped = 0;
    if (i < n) v[i] = 0.0;
}

// Entry (r, c) of the pattern, or -1. The row's range is clipped to [0, nnz),
// so a malformed rowptr cannot send the search outside col.
__device__ __forceinline__ int find_entry(const int32_t *rowptr, const int32_t *col, int nnz, int r, int c) {
    int lo = max(rowptr[r], 0), hi = min(rowptr[r + 1], nnz) - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int v = col[mid];
        if (v == c) return mid;
        if (v < c) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// Adds each face's halves into both directions of its three edges
// (arap.h:225-232). An edge of a manifold mesh receives at most two additions
// onto zero, which round the same in either order. A face whose corners
// repeat a vertex gives a diagonal entry both directions' halves, as the
// reference's two triplets (a, a) do. Faces with an out-of-range index are
// skipped (counted by k_face_cots_to_scratch); an edge missing from the
// pattern is counted here.
__global__ void k_scatter_weights(int F, int V, int nnz, const int32_t *__restrict__ faces,
                                  const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                                  const double *__restrict__ hc, double *__restrict__ val, int *skipped) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * F) return;
    const int f = t / 3, k = t - 3 * f;
    const int i0 = faces[3 * f], i1 = faces[3 * f + 1], i2 = faces[3 * f + 2];
    if (!in_range(i0, V) || !in_range(i1, V) || !in_range(i2, V)) return;
    const int a = faces[3 * f + k], b = faces[3 * f + (k + 1) % 3];
    const double h = hc[t];
    const int e1 = find_entry(rowptr, col, nnz, a, b);
    const int e2 = find_entry(rowptr, col, nnz, b, a);
    if (e1 >= 0) atomicAdd(val + e1, h);
    if (e2 >= 0) atomicAdd(val + e2, h);
    if (e1 < 0 || e2 < 0) atomicAdd(skipped, 1);
}

}  // namespace

extern "C" int arap_cotan_weights_static(int32_t n_vertices, int32_t n_faces, const int32_t *faces,
                                         const double *xyz, const int32_t *rowptr, const int32_t *col, int32_t nnz,
                                         double *val, void *stream) {
    if (n_vertices < 0 || n_faces < 0 || nnz < 0 || (n_faces > 0 && (!faces || !xyz || !rowptr || !col)) ||
        (nnz > 0 && !val)) {
        arapgpu::set_global_error("arap_cotan_weights_static: invalid argument");
        return ARAP_ERR_INVALID_ARGUMENT;
    }
    if (n_faces > kStaticMaxFaces) {
        arapgpu::set_global_error("arap_cotan_weights_static: " + std::to_string(n_faces) +
                                  " faces exceed the static scratch limit of " + std::to_string(kStaticMaxFaces));
        return ARAP_ERR_UNSUPPORTED;
    }
    int device = 0;
    if (current_device(&device) != ARAP_OK) {
        arapgpu::set_global_error("arap_cotan_weights_static: no usable current device");
        return ARAP_ERR_NO_DEVICE;
    }
    double *hc = nullptr;
    int *skipped = nullptr;
    cudaError_t e = symbol_addresses(device, &hc, &skipped);
    if (e != cudaSuccess) {
        arapgpu::set_global_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return ARAP_ERR_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_zero<<<(nnz + 255) / 256 + (nnz == 0), 256, 0, st>>>(nnz, val, skipped);
    if (n_faces > 0) {
        k_face_cots_to_scratch<<<(n_faces + 255) / 256, 256, 0, st>>>(n_faces, n_vertices, faces, xyz, hc, skipped);
        k_scatter_weights<<<(3 * n_faces + 255) / 256, 256, 0, st>>>(n_faces, n_vertices, nnz, faces, rowptr, col,
                                                                      hc, val, skipped);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        arapgpu::set_global_error(std::string("arap_cotan_weights_static launch: ") + cudaGetErrorString(e));
        return ARAP_ERR_CUDA;
    }
    return ARAP_OK;
}

extern "C" int arap_cotan_weights_static_status(void *stream, int32_t *skipped) {
    int device = 0;
    if (current_device(&device) != ARAP_OK) {
        arapgpu::set_global_error("arap_cotan_weights_static_status: no usable current device");
        return ARAP_ERR_NO_DEVICE;
    }
    double *hc = nullptr;
    int *counter = nullptr;
    cudaError_t e = symbol_addresses(device, &hc, &counter);
    int n = 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&n, counter, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        arapgpu::set_global_error(std::string("arap_cotan_weights_static_status: ") + cudaGetErrorString(e));
        return ARAP_ERR_CUDA;
    }
    if (skipped) *skipped = n;
    if (n > 0) {
        arapgpu::set_global_error("arap_cotan_weights_static: " + std::to_string(n) +
                                  " faces with an index outside [0, n_vertices) or edges missing from the pattern");
        return ARAP_ERR_BAD_INDEX;
    }
    return ARAP_OK;
}
