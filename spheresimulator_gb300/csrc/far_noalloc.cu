// far_noalloc.cu — traction far field that allocates no device memory.
//
// Some callers of this library cannot call cudaMalloc at the point where they need the far
// field: a host application that has already reserved (nearly) all of the GPU's memory for its
// own pool allocator leaves nothing for the library to allocate, and a solver loop that applies
// the operator thousands of times (the collision complementarity iterations around the mobility
// operator) cannot afford cudaMalloc/cudaFree there, since cudaFree synchronizes the whole device.
// This entry point therefore takes every input and output from the caller as device pointers and
// keeps its only scratch — the per-chunk partial sums of the split source loop — in a file-scope
// __device__ array of fixed size. Every GPU that loads the library holds that array
// (kNoAllocMaxPoints * kNoAllocChunks * 3 doubles = 7.5 MiB) until the process exits.
//
// The kernel is a variant of k_far64 (farfield.cu): targets in blocks of 128, the sources of all
// points split into kNoAllocChunks fixed ranges, pairs on the target's own sphere skipped, partial
// sums per chunk reduced in a fixed order afterwards. Unlike the context entry points it has no
// neighbour list, so near-pair spheres are not excluded: the result is the smooth-quadrature
// traction of every point on another sphere (the far-field part of
// BIE/SphereSTKSHOperator.cpp:368-446 after its own-sphere subtraction).
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/smob.h"
#include "smob_internal.h"

namespace smob {
void set_last_error(const char* msg);
}

namespace {

constexpr int kNoAllocMaxPoints = 40960;
constexpr int kNoAllocChunks = 8;
constexpr int kNoAllocThreads = 128;
constexpr int kNoAllocTile = 128;
constexpr int kNoAllocMaxDevices = 64;

// Shared by every call on a device; it keeps the previous call's partial sums. Nothing in it
// needs to start at zero: each call writes every entry it later reads (all chunks x all targets).
static __device__ __align__(256) double g_far_noalloc_scratch[kNoAllocChunks * kNoAllocMaxPoints * 3];

// Scratch addresses looked up so far, one per (device, CUDA context): the address of a __device__
// array belongs to the context that loaded the module, so a non-primary context on the same device,
// or the primary context created again after cudaDeviceReset, has its own.
struct ScratchAddr {
    int dev;
    void* ctx;
    double* addr;
};
std::mutex g_setup_mu;
ScratchAddr g_scratch_addr[kNoAllocMaxDevices] = {};
int g_scratch_count = 0;

__global__ void __launch_bounds__(kNoAllocThreads)
    k_far_noalloc_partial(const double* __restrict__ coords, const double* __restrict__ norms,
                          const double* __restrict__ weights, const double* __restrict__ density,
                          const int* __restrict__ sphere, int n, double c, double* __restrict__ partial) {
    __shared__ double sp[3 * kNoAllocTile];
    __shared__ double sf[3 * kNoAllocTile];
    __shared__ int ss[kNoAllocTile];
    const int chunk = blockIdx.y;
    const int t = blockIdx.x * kNoAllocThreads + threadIdx.x;
    const bool valid = t < n;
    const long long s0 = (long long)chunk * n / kNoAllocChunks, s1 = (long long)(chunk + 1) * n / kNoAllocChunks;
    double tx = 0, ty = 0, tz = 0, nx = 0, ny = 0, nz = 0;
    int sid = -1;
    if (valid) {
        tx = coords[3 * t];
        ty = coords[3 * t + 1];
        tz = coords[3 * t + 2];
        nx = norms[3 * t];
        ny = norms[3 * t + 1];
        nz = norms[3 * t + 2];
        sid = sphere[t];
    }
    double ax = 0, ay = 0, az = 0;
    for (long long base = s0; base < s1; base += kNoAllocTile) {
        const int m = (int)min((long long)kNoAllocTile, s1 - base);
        __syncthreads();
        for (int k = threadIdx.x; k < m; k += kNoAllocThreads) {
            const long long j = base + k;
            const double w = weights[j] * c;
            sp[3 * k] = coords[3 * j];
            sp[3 * k + 1] = coords[3 * j + 1];
            sp[3 * k + 2] = coords[3 * j + 2];
            sf[3 * k] = density[3 * j] * w;
            sf[3 * k + 1] = density[3 * j + 1] * w;
            sf[3 * k + 2] = density[3 * j + 2] * w;
            ss[k] = sphere[j];
        }
        __syncthreads();
        if (valid) {
            for (int k = 0; k < m; ++k) {
                if (ss[k] == sid) continue;
                const double rx = tx - sp[3 * k], ry = ty - sp[3 * k + 1], rz = tz - sp[3 * k + 2];
                const double r2 = rx * rx + ry * ry + rz * rz;
                if (r2 == 0) continue;  // a point of another sphere at the target itself adds nothing
                const double ri = rsqrt(r2);
                const double ri2 = ri * ri;
                const double rf = rx * sf[3 * k] + ry * sf[3 * k + 1] + rz * sf[3 * k + 2];
                const double rn = rx * nx + ry * ny + rz * nz;
                const double q = rf * rn * ri2 * ri2 * ri;
                ax += q * rx;
                ay += q * ry;
                az += q * rz;
            }
        }
    }
    if (valid) {
        double* o = partial + ((long long)chunk * n + t) * 3;
        o[0] = ax;
        o[1] = ay;
        o[2] = az;
    }
}

__global__ void k_far_noalloc_reduce(const double* __restrict__ partial, int n, double pre, double* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double sx = 0, sy = 0, sz = 0;
    for (int c = 0; c < kNoAllocChunks; ++c) {
        const double* q = partial + ((long long)c * n + t) * 3;
        sx += q[0];
        sy += q[1];
        sz += q[2];
    }
    out[3 * t] += pre * sx;
    out[3 * t + 1] += pre * sy;
    out[3 * t + 2] += pre * sz;
}

// The current CUDA context (driver cuCtxGetCurrent, reached through the runtime so that the library
// does not link libcuda); nullptr if it cannot be queried.
void* current_context() {
    using Fn = int (*)(void**);
    static Fn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return reinterpret_cast<Fn>(f);
    }();
    void* ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

// Device address of the scratch array in the current context. Host code cannot use the symbol
// itself as a pointer (it names a host-side shadow). Outside stream capture the address is looked
// up with cudaGetSymbolAddress on every call (a lookup in the runtime's table once the module is
// loaded), so a reset device or another context gets its own address; during capture, where that
// call may have to load the module, the address cached for the current (device, context) is used,
// and a context without one is refused.
smob_status scratch_for_call(cudaStream_t st, double** ptr) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        cudaGetLastError();
        smob::set_last_error("smob_far_traction_noalloc: no usable current CUDA device");
        return SMOB_ERR_NO_DEVICE;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    bool capturing = false;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        cudaGetLastError();
        capturing = true;  // the legacy stream while another thread captures: treat as capture
    } else {
        capturing = cs != cudaStreamCaptureStatusNone;
    }
    void* ctx = current_context();
    std::lock_guard<std::mutex> lk(g_setup_mu);
    ScratchAddr* slot = nullptr;
    for (int i = 0; i < g_scratch_count; ++i)
        if (g_scratch_addr[i].dev == dev && g_scratch_addr[i].ctx == ctx) slot = &g_scratch_addr[i];
    if (!capturing) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_far_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            smob::set_last_error("smob_far_traction_noalloc: cudaGetSymbolAddress of the scratch array failed");
            return SMOB_ERR_CUDA;
        }
        if (!slot) {
            // full table (more contexts than kNoAllocMaxDevices): reuse the oldest entry
            slot = &g_scratch_addr[g_scratch_count < kNoAllocMaxDevices ? g_scratch_count++ : 0];
            slot->dev = dev;
            slot->ctx = ctx;
        }
        slot->addr = static_cast<double*>(p);
    } else if (!slot) {
        smob::set_last_error("smob_far_traction_noalloc: the first call in a CUDA context must come before any "
                             "stream capture (it looks up the scratch array's device address)");
        return SMOB_ERR_STATE;
    }
    *ptr = slot->addr;
    return SMOB_OK;
}

}  // namespace

extern "C" smob_status smob_far_traction_noalloc(const double* d_coords, const double* d_norms, const double* d_weights,
                                                 const double* d_density, const int* d_sphere, int n_points, double c,
                                                 double* d_out, void* stream) {
    if (n_points < 1 || n_points > kNoAllocMaxPoints) {
        smob::set_last_error("smob_far_traction_noalloc: n_points must be in [1, 40960] (the fixed scratch size)");
        return SMOB_ERR_ARG;
    }
    if (!d_coords || !d_norms || !d_weights || !d_density || !d_sphere || !d_out) {
        smob::set_last_error("smob_far_traction_noalloc: null device pointer");
        return SMOB_ERR_ARG;
    }
    double* scratch = nullptr;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const smob_status s = scratch_for_call(st, &scratch);
    if (s != SMOB_OK) return s;
    const dim3 grid((n_points + kNoAllocThreads - 1) / kNoAllocThreads, kNoAllocChunks);
    k_far_noalloc_partial<<<grid, kNoAllocThreads, 0, st>>>(d_coords, d_norms, d_weights, d_density, d_sphere, n_points,
                                                            c, scratch);
    k_far_noalloc_reduce<<<(n_points + 255) / 256, 256, 0, st>>>(scratch, n_points, -3.0 / (4 * 3.14159265358979323846),
                                                                 d_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        smob::set_last_error(cudaGetErrorString(e));
        return SMOB_ERR_CUDA;
    }
    return SMOB_OK;
}
