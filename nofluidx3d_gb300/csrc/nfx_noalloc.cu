// nfx_indenter_force_noalloc: the indenter-force readout for callers that cannot allocate
// device memory.
//
// The readout of nfx_indenter_force reduces one value per node in a fixed order through
// per-block partial sums and a completion counter; in the handle those live in device memory
// the library allocated. Some callers hold positions in their own device buffers and are not
// allowed to allocate at all: a host solver that carves every byte of device memory out of its
// own pool at start-up and forbids cudaMalloc afterwards, or a coupling layer that calls into
// this library from a time loop where an allocation (and the device synchronisation it can
// imply) is not acceptable. For them this entry point keeps its scratch in a file-scope
// static device array of fixed size: the partial sums of at most NOALLOC_MAX_BLOCKS blocks of
// 256 nodes (128 KiB) plus the counter. Every GPU that loads the library holds the array
// until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/nfx.h"
#include "nfx_internal.h"

namespace {

constexpr int NOALLOC_BLOCK = 256;
constexpr long long NOALLOC_MAX_BLOCKS = 16384;
constexpr long long NOALLOC_MAX_NODES = NOALLOC_MAX_BLOCKS * NOALLOC_BLOCK;  // 4,194,304
constexpr int NOALLOC_TAIL = 32;  // 256 bytes after the partials; the counter sits in the first word

// The shared scratch: partial sums, then the completion counter. Contents persist between
// calls; the counter is cleared at the start of every call.
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_MAX_BLOCKS + NOALLOC_TAIL];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[MAX_DEVICES] = {nullptr};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Same contact laws and sign as the handle's readout: the force the cell exerts on the contact
// along y (Simulation.py:146-153 plane, :198-212 sphere), i.e. minus the y force on the nodes.
__global__ void __launch_bounds__(NOALLOC_BLOCK) k_readout_noalloc(long long np, const double* __restrict__ pts,
                                                                   int kind, double k, double radius, double w,
                                                                   double* scratch, double* out) {
    __shared__ double s_w[NOALLOC_BLOCK / 32];
    __shared__ int s_last;
    const long long i = (long long)blockIdx.x * NOALLOC_BLOCK + threadIdx.x;
    double ro = 0.0;
    if (i < np) {
        const double y = pts[np + i];
        if (kind == NFX_CONTACT_SUBSTRATE) {
            ro = -(k * fmax(w - y, 0.0));
        } else if (kind == NFX_CONTACT_PLANE) {
            ro = k * fmax(y - w, 0.0);
        } else {
            const double rx = pts[i], ry = y - w, rz = pts[2 * np + i];
            const double len = sqrt(rx * rx + ry * ry + rz * rz);
            const double dis = fmax(radius - len, 0.0);
            if (dis != 0.0) ro = -((k * dis) * (ry / len));
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ro = warp_sum(ro);
    if (lane == 0) s_w[warp] = ro;
    __syncthreads();
    unsigned* counter = reinterpret_cast<unsigned*>(scratch + NOALLOC_MAX_BLOCKS);
    if (warp == 0) {
        double x = lane < NOALLOC_BLOCK / 32 ? s_w[lane] : 0.0;
        x = warp_sum(x);
        if (lane == 0) {
            scratch[blockIdx.x] = x;
            __threadfence();
            s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const volatile double* part = scratch;
    double acc = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += NOALLOC_BLOCK) acc += part[b];
    acc = warp_sum(acc);
    if (lane == 0) s_w[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int q = 0; q < NOALLOC_BLOCK / 32; q++) tot += s_w[q];
        *out = tot;
        *counter = 0u;
    }
}

// The device address of the static scratch in the current context of device `dev`. The address
// is looked up again on every call made outside stream capture, so a context that was reset
// (cudaDeviceReset) or a different context made current since the last call gets its own
// module's address; inside a capture the address cached by the last uncaptured call is used.
int scratch_for_device(int dev, cudaStream_t st, double** ptr) {
    if (dev < 0 || dev >= MAX_DEVICES) {
        nfx::set_error("device index out of range for the no-alloc scratch table");
        return NFX_ERR_ARG;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const cudaError_t ce = cudaStreamIsCapturing(st, &cap);
    const bool capturing = ce != cudaSuccess || cap != cudaStreamCaptureStatusNone;
    if (ce != cudaSuccess) cudaGetLastError();  // e.g. the legacy stream during another stream's capture
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!capturing) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            nfx::set_error(std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
            return NFX_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<double*>(p);
    } else if (!g_scratch_ptr[dev]) {
        nfx::set_error("the first nfx_indenter_force_noalloc call on a device must come before any stream capture");
        return NFX_ERR_STATE;
    }
    *ptr = g_scratch_ptr[dev];
    return NFX_OK;
}

// Makes `dev` current for the lifetime of the guard and gives the caller its own current
// device back afterwards.
struct DeviceGuard {
    int prev = -1;
    bool switched = false;
    cudaError_t enter(int dev) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return e;
        if (prev == dev) return cudaSuccess;
        e = cudaSetDevice(dev);
        switched = e == cudaSuccess;
        return e;
    }
    ~DeviceGuard() {
        if (switched) cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" int nfx_indenter_force_noalloc(int device, int64_t np, const double* points_dev, int kind, double k,
                                          double radius, double position, double* out_dev, void* stream) {
    if (!points_dev || !out_dev) {
        nfx::set_error("null device pointer");
        return NFX_ERR_ARG;
    }
    if (np <= 0 || np > NOALLOC_MAX_NODES) {
        nfx::set_error("np = " + std::to_string((long long)np) + " is outside 1.." + std::to_string(NOALLOC_MAX_NODES) +
                        ", the node count the static scratch of nfx_indenter_force_noalloc supports");
        return NFX_ERR_ARG;
    }
    if (kind != NFX_CONTACT_SUBSTRATE && kind != NFX_CONTACT_PLANE && kind != NFX_CONTACT_SPHERE) {
        nfx::set_error("unknown contact kind");
        return NFX_ERR_ARG;
    }
    if (!std::isfinite(k) || !std::isfinite(radius) || !std::isfinite(position)) {
        nfx::set_error("non-finite contact parameter");
        return NFX_ERR_ARG;
    }
    DeviceGuard guard;
    cudaError_t e = guard.enter(device);
    if (e != cudaSuccess) {
        nfx::set_error(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        return NFX_ERR_NODEVICE;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double* scratch = nullptr;
    int rc = scratch_for_device(device, st, &scratch);
    if (rc != NFX_OK) return rc;
    // the counter must start at zero; clear it in stream order
    e = cudaMemsetAsync(scratch + NOALLOC_MAX_BLOCKS, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) {
        nfx::set_error(std::string("cudaMemsetAsync(counter): ") + cudaGetErrorString(e));
        return NFX_ERR_CUDA;
    }
    const unsigned blocks = (unsigned)((np + NOALLOC_BLOCK - 1) / NOALLOC_BLOCK);
    k_readout_noalloc<<<blocks, NOALLOC_BLOCK, 0, st>>>((long long)np, points_dev, kind, k, radius, position, scratch,
                                                        out_dev);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        nfx::set_error(std::string("k_readout_noalloc launch: ") + cudaGetErrorString(e));
        return NFX_ERR_CUDA;
    }
    return NFX_OK;
}
