// noalloc.cu -- eu_totals_noalloc: the conserved-totals audit (eu_totals) for
// callers that cannot let this library allocate device memory.
//
// Who needs it: a caller that owns all device memory through its own pool
// (a framework's caching allocator, an application that reserves the whole
// HBM at start-up, a real-time loop in which cudaMalloc/cudaFree -- which can
// synchronise the device and fragment the pool -- are not allowed).  Such a
// caller has its grid in device memory already and cannot create an
// eu_handle, because eu_create allocates the state, workspace and control
// block.  This entry point takes the caller's device grid and device output
// pointer and allocates nothing: no cudaMalloc/cudaFree, no allocating
// library.
//
// Scratch: the per-row partial sums live in g_row_part below, a fixed-size
// array in this library's own device image (kNoallocMaxRows rows x 8 doubles
// = 1 MiB).  Grids with more than kNoallocMaxRows interior rows are rejected
// with EU_ERR_INVALID.  Nothing in the scratch has to start at zero: pass 1
// writes the slots of rows 0..ny-1 before pass 2 reads exactly those slots.
//
// Set-up: every call looks the scratch address up with cudaGetSymbolAddress,
// with the calling thread's current device current, checks the result and
// passes that address to the kernels.  The host-side name g_row_part is only
// a stand-in for the device array and is never handed to a kernel.  The
// lookup is repeated on every call instead of being cached, because after a
// cudaDeviceReset (or any re-creation of the primary context) the library's
// device image is loaded again, possibly at another address, and a cached
// address would make the kernels write through a stale pointer.  With lazy
// module loading (the CUDA default) the first call on a device also loads
// this library's device image, including the 1 MiB array, so that first
// call may take device memory once; callers that hand all HBM to their own
// pool should make one warm-up call (or set CUDA_MODULE_LOADING=EAGER)
// before they reserve it, and make the first call before any stream capture
// begins.
//
// Concurrency: every call on one device uses the same scratch.  Two calls
// whose work overlaps on the device (different streams, or different host
// threads, without ordering between them) race on the scratch and give wrong
// totals.  Order them on one stream or with events.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/euler2d.h"

namespace eu {
void set_global_error(const char* msg);
}

namespace {

constexpr int kNoallocMaxRows = 16384;
constexpr int kRowsPerBlock = 8;  // one warp per interior row

// Row partials: row j's Neumaier sum of field f at [8j + f], its
// compensation at [8j + 4 + f].
static __device__ __align__(256) double g_row_part[kNoallocMaxRows * 8];

__device__ __forceinline__ void two_sum_add(double& s, double& c, double x) {
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
}

// Pass 1: warp w of block b sums interior row j = 8b + w (AoS row j + 2,
// columns 2..nx+1) with per-lane Neumaier sums, folds the lanes in a fixed
// shuffle order and writes the row's pair to part.
__global__ void __launch_bounds__(32 * kRowsPerBlock) noalloc_rows_kernel(const double* __restrict__ aos, int nx,
                                                                          int ny, double* __restrict__ part) {
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * kRowsPerBlock + (threadIdx.x >> 5);
    if (j >= ny) return;
    const long long tnx = nx + 4;
    const double2* row = reinterpret_cast<const double2*>(aos + 4 * ((j + 2) * tnx + 2));
    double s[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0};
    for (int i = lane; i < nx; i += 32) {
        const double2 a = row[2 * i], b = row[2 * i + 1];
        two_sum_add(s[0], c[0], a.x);
        two_sum_add(s[1], c[1], a.y);
        two_sum_add(s[2], c[2], b.x);
        two_sum_add(s[3], c[3], b.y);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const double so = __shfl_down_sync(0xffffffffu, s[f], off);
            const double co = __shfl_down_sync(0xffffffffu, c[f], off);
            two_sum_add(s[f], c[f], so);
            c[f] += co;
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            part[8 * j + f] = s[f];
            part[8 * j + 4 + f] = c[f];
        }
    }
}

// Pass 2: one block of 4 x 64 threads; thread (f, k) folds rows k, k+64, ...
// of field f, then thread (f, 0) folds the 64 results in order.
__global__ void __launch_bounds__(256) noalloc_fold_kernel(const double* __restrict__ part, int ny,
                                                           double* __restrict__ out) {
    __shared__ double sh[4][64], shc[4][64];
    const int f = threadIdx.x >> 6, k = threadIdx.x & 63;
    double s = 0.0, c = 0.0;
    for (int j = k; j < ny; j += 64) {
        two_sum_add(s, c, part[8 * j + f]);
        c += part[8 * j + 4 + f];
    }
    sh[f][k] = s;
    shc[f][k] = c;
    __syncthreads();
    if (k == 0) {
        double a = 0.0, ac = 0.0;
        for (int q = 0; q < 64; ++q) {
            two_sum_add(a, ac, sh[f][q]);
            ac += shc[f][q];
        }
        out[f] = a + ac;
    }
}

int fail(int code, const char* msg) {
    eu::set_global_error(msg);
    return code;
}

// Is p a device pointer of the current device (or managed memory)?
bool on_device(const void* p, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" int eu_totals_noalloc(const double* d_aos, int nx, int ny, double* d_out, void* stream) {
    if (!d_aos || !d_out) return fail(EU_ERR_INVALID, "eu_totals_noalloc: null pointer");
    if (nx < 1 || ny < 1) return fail(EU_ERR_INVALID, "eu_totals_noalloc: nx and ny must be >= 1");
    if (ny > kNoallocMaxRows)
        return fail(EU_ERR_INVALID,
                    "eu_totals_noalloc: ny exceeds the fixed scratch of 16384 interior rows; "
                    "use eu_totals on a handle for larger grids");
    if ((reinterpret_cast<uintptr_t>(d_aos) & 15u) || (reinterpret_cast<uintptr_t>(d_out) & 7u))
        return fail(EU_ERR_INVALID, "eu_totals_noalloc: d_aos must be 16-byte and d_out 8-byte aligned");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        (void)cudaGetLastError();
        return fail(EU_ERR_CUDA, "eu_totals_noalloc: no usable current CUDA device");
    }
    if (!on_device(d_aos, dev) || !on_device(d_out, dev))
        return fail(EU_ERR_INVALID, "eu_totals_noalloc: d_aos and d_out must be device memory of the current device");
    // the scratch's device address in the current context (see the header)
    void* p = nullptr;
    const cudaError_t le = cudaGetSymbolAddress(&p, g_row_part);
    if (le != cudaSuccess || !p) {
        (void)cudaGetLastError();
        return fail(EU_ERR_CUDA, "eu_totals_noalloc: cudaGetSymbolAddress of the scratch failed");
    }
    double* scratch = static_cast<double*>(p);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int blocks = (ny + kRowsPerBlock - 1) / kRowsPerBlock;
    noalloc_rows_kernel<<<blocks, 32 * kRowsPerBlock, 0, s>>>(d_aos, nx, ny, scratch);
    noalloc_fold_kernel<<<1, 256, 0, s>>>(scratch, ny, d_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(EU_ERR_CUDA, cudaGetErrorString(e));
    return EU_OK;
}
