// ref_gpu_harness.cu -- runs the reference's OWN CUDA kernels on this GPU
// (comparison timing and test infrastructure: never part of the product).
//
// The reference's GPU solver (src/gpu/solver_gpu.cu) is compiled, unmodified,
// from its own sources into a device image (oracle/_ref/ref_solver_gpu.cubin,
// `make -C oracle refgpu` on the build host, where the reference tree lies).
// Its host-side code cannot be built on the GPU host (the sources are not
// there, and objects built elsewhere are for another CPU), so this harness
// loads the device image with the driver API and replays the host side of
// the reference's GPU time loop:
//   scripts/gpu/main_gpu.cu:242-266        per step: compute_dt_gpu, t_end clip,
//                                          advance_second_order_gpu, swap
//   src/gpu/solver_gpu.cu:741-782          compute_dt_gpu: block-max kernel
//                                          (256 threads), a device max over the
//                                          block maxima (CUB DeviceReduce::Max,
//                                          as the reference), an 8-byte copy to
//                                          the host, cfl*min(dx,dy)/max
//   src/gpu/solver_gpu.cu:818-885          advance_second_order_gpu: the x and
//                                          y fused kernels on 16x16 blocks with
//                                          the reference's shared-memory sizes
// The kernels are found by name in the image (their symbols carry the
// reference's own mangled names) and launched with the reference's argument
// layout (head/gpu/grid_gpu.cuh:156-188, Grid2DGPUView / ConstGrid2DGPUView;
// head/riemann.hpp:13-18, RiemannSolver).
#include <cub/cub.cuh>
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <cxxabi.h>
#include <cstdlib>
#include <string>
#include <vector>

namespace {

// Argument layout of the reference's grid views (head/gpu/grid_gpu.cuh:156-188).
struct View {
    int nx, ny, ng;
    double x_min, x_max, y_min, y_max, dx, dy;
    double *rho, *rhou, *rhov, *E;
};

struct Grid {
    double* f[4] = {nullptr, nullptr, nullptr, nullptr};
};

char g_err[512];

int fail(const char* what, int code) {
    std::snprintf(g_err, sizeof(g_err), "%s (%d)", what, code);
    return 1;
}

#define DRV(call)                                          \
    do {                                                   \
        CUresult r_ = (call);                              \
        if (r_ != CUDA_SUCCESS) return fail(#call, (int)r_); \
    } while (0)
#define RT(call)                                           \
    do {                                                   \
        cudaError_t r_ = (call);                           \
        if (r_ != cudaSuccess) return fail(#call, (int)r_); \
    } while (0)

// The image's kernel whose demangled name contains `key`.
int find_kernel(CUmodule mod, const char* key, CUfunction* out) {
    unsigned int n = 0;
    DRV(cuModuleGetFunctionCount(&n, mod));
    std::vector<CUfunction> fs(n);
    DRV(cuModuleEnumerateFunctions(fs.data(), n, mod));
    for (CUfunction f : fs) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
        int st = 0;
        char* dem = abi::__cxa_demangle(name, nullptr, nullptr, &st);
        const bool hit = std::strstr(dem ? dem : name, key) != nullptr;
        std::free(dem);
        if (hit) {
            *out = f;
            return 0;
        }
    }
    std::snprintf(g_err, sizeof(g_err), "kernel %s not found in the reference image", key);
    return 1;
}

View view_of(const Grid& g, int nx, int ny, double x0, double x1, double y0, double y1) {
    View v;
    v.nx = nx; v.ny = ny; v.ng = 2;
    v.x_min = x0; v.x_max = x1; v.y_min = y0; v.y_max = y1;
    v.dx = (x1 - x0) / (double)nx;   // head/gpu/grid_gpu.cuh: Grid2DGPU::allocate
    v.dy = (y1 - y0) / (double)ny;
    v.rho = g.f[0]; v.rhou = g.f[1]; v.rhov = g.f[2]; v.E = g.f[3];
    return v;
}

}  // namespace

extern "C" {

const char* refgpu_last_error(void) { return g_err; }

// Runs `warmup` + `nsteps` steps of the reference's GPU time loop (free CFL
// steps, no t_end clip) on the AoS grid `aos` (Grid2D layout, 4 doubles per
// cell, ghosts included; the reference's kernels clamp their stencil at the
// domain edge, so ghost values are not read), and writes the final state
// back into `aos` (interior; ghosts by the transmissive rule).
//   image    path of the reference's device image
//   ms       out, 4 values over the timed steps: wall-clock ms of the whole
//            loop (the reference's per-step host synchronisation included),
//            then the summed device ms of the dt kernel + reduction, the x
//            kernel and the y kernel (CUDA events)
//   dts      out (may be NULL): the nsteps timed step sizes
// Returns 0, or 1 with refgpu_last_error() set.
int refgpu_run(const char* image, double* aos, int nx, int ny, double x0, double x1, double y0, double y1,
               int solver, double cfl, int warmup, int nsteps, double* ms, double* dts) {
    g_err[0] = 0;
    RT(cudaFree(nullptr));   // the runtime's primary context, current on this thread
    CUmodule mod = nullptr;
    DRV(cuModuleLoad(&mod, image));
    CUfunction kdt, kx, ky;
    if (find_kernel(mod, "compute_block_max_speed_kernel<256>", &kdt) ||
        find_kernel(mod, "advance_x_reconstruct_smem_fused_kernel", &kx) ||
        find_kernel(mod, "advance_y_reconstruct_smem_fused_kernel", &ky)) {
        cuModuleUnload(mod);
        return 1;
    }
    const int tnx = nx + 4, tny = ny + 4;
    const size_t cells = (size_t)tnx * tny;
    Grid G[3];
    for (auto& g : G)
        for (int f = 0; f < 4; ++f) RT(cudaMalloc(&g.f[f], cells * sizeof(double)));
    // upload: AoS -> the reference's SoA planes (head/gpu/grid_gpu.cuh:90-104)
    {
        std::vector<double> plane(cells);
        for (int f = 0; f < 4; ++f) {
            for (size_t k = 0; k < cells; ++k) plane[k] = aos[4 * k + f];
            RT(cudaMemcpy(G[0].f[f], plane.data(), cells * sizeof(double), cudaMemcpyHostToDevice));
        }
    }
    // compute_dt_gpu workspace (src/gpu/solver_gpu.cu:691-719)
    const int interior = nx * ny;
    const int nblk = (interior + 255) / 256;
    double *speed = nullptr, *maxd = nullptr;
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
    RT(cudaMalloc(&speed, (size_t)nblk * sizeof(double)));
    RT(cudaMalloc(&maxd, sizeof(double)));
    RT(cub::DeviceReduce::Max(nullptr, tmp_bytes, speed, maxd, nblk));
    RT(cudaMalloc(&tmp, tmp_bytes));
    // advance_second_order_gpu launch shape (src/gpu/solver_gpu.cu:830-884)
    const unsigned bx = (unsigned)(nx + 15) / 16, by = (unsigned)(ny + 15) / 16;
    const size_t smem_x = (4 * (size_t)(16 + 4 + 1) * 16 + 8 * (size_t)(16 + 2 + 1) * 16 + 4 * (size_t)(16 + 1) * 16) *
                          sizeof(double);
    const size_t smem_y = (4 * (size_t)(16 + 1) * (16 + 4) + 8 * (size_t)(16 + 1) * (16 + 2) +
                           4 * (size_t)(16 + 1) * (16 + 1)) * sizeof(double);
    cudaEvent_t ev[6];
    for (auto& e : ev) RT(cudaEventCreate(&e));
    float acc[3] = {0.f, 0.f, 0.f};
    int cur = 0, mid = 1, nxt = 2;
    double wall_ms = 0.0;
    for (int s = 0; s < warmup + nsteps; ++s) {
        const bool timed = s >= warmup;
        const auto t0 = std::chrono::steady_clock::now();
        View vu = view_of(G[cur], nx, ny, x0, x1, y0, y1);
        View vm = view_of(G[mid], nx, ny, x0, x1, y0, y1);
        View vn = view_of(G[nxt], nx, ny, x0, x1, y0, y1);
        RT(cudaEventRecord(ev[0], 0));
        {
            void* args[] = {&vu, &speed};
            DRV(cuLaunchKernel(kdt, (unsigned)nblk, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr));
        }
        RT(cub::DeviceReduce::Max(tmp, tmp_bytes, speed, maxd, nblk));
        RT(cudaEventRecord(ev[1], 0));
        double smax = 0.0;
        RT(cudaMemcpy(&smax, maxd, sizeof(double), cudaMemcpyDeviceToHost));
        double dt = smax <= 0.0 ? 1.0e300 : cfl * std::min(vu.dx, vu.dy) / smax;
        double dt_arg = dt;
        int sol = solver;
        RT(cudaEventRecord(ev[2], 0));
        {
            void* args[] = {&vu, &vm, &dt_arg, &sol};
            DRV(cuLaunchKernel(kx, bx, by, 1, 16, 16, 1, (unsigned)smem_x, nullptr, args, nullptr));
        }
        RT(cudaEventRecord(ev[3], 0));
        {
            void* args[] = {&vm, &vn, &dt_arg, &sol};
            DRV(cuLaunchKernel(ky, bx, by, 1, 16, 16, 1, (unsigned)smem_y, nullptr, args, nullptr));
        }
        RT(cudaEventRecord(ev[4], 0));
        RT(cudaEventSynchronize(ev[4]));
        const auto t1 = std::chrono::steady_clock::now();
        if (timed) {
            wall_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
            float a = 0.f, b = 0.f, c = 0.f;
            RT(cudaEventElapsedTime(&a, ev[0], ev[1]));
            RT(cudaEventElapsedTime(&b, ev[2], ev[3]));
            RT(cudaEventElapsedTime(&c, ev[3], ev[4]));
            acc[0] += a; acc[1] += b; acc[2] += c;
            if (dts) dts[s - warmup] = dt;
        }
        std::swap(cur, nxt);   // d_U.swap(d_U_next)
    }
    ms[0] = wall_ms;
    ms[1] = acc[0];
    ms[2] = acc[1];
    ms[3] = acc[2];
    // download into the AoS grid, ghosts by the transmissive rule
    {
        std::vector<double> plane(cells);
        for (int f = 0; f < 4; ++f) {
            RT(cudaMemcpy(plane.data(), G[cur].f[f], cells * sizeof(double), cudaMemcpyDeviceToHost));
            for (int j = 0; j < tny; ++j)
                for (int i = 0; i < tnx; ++i) {
                    const int si = std::min(std::max(i, 2), nx + 1), sj = std::min(std::max(j, 2), ny + 1);
                    aos[4 * ((size_t)j * tnx + i) + f] = plane[(size_t)sj * tnx + si];
                }
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    cudaFree(speed); cudaFree(maxd); cudaFree(tmp);
    for (auto& g : G)
        for (int f = 0; f < 4; ++f) cudaFree(g.f[f]);
    cuModuleUnload(mod);
    return 0;
}

}  // extern "C"
