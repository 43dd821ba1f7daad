"""The FP32 form's p*/u* route of the exact Riemann solver (exact_star_mixed
in large_sys_eq_opt_gb300/csrc/euler_numerics.cuh: Newton's iteration in
FP32, one FP64 Newton step, u* from the linearised FP64 pressure
functions)
against the FP64 iteration that the FP64 form runs (exact_star, after
head/riemann.hpp:361-443), on the same FP32 face states: random Riemann
problems with pressure ratios up to 1e6, strong shocks, strong
rarefactions, near-vacuum and vacuum-generating states and identical
pressures.  Where the FP64 iteration converges, both agree to 1e-10 relative
in p* and u*; where the FP64 iteration halves toward vacuum, the mixed
route hands over to it and returns its bits."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "large_sys_eq_opt_gb300", "csrc")

SRC = r"""
#include <cstdio>
#include <cuda_runtime.h>
#include "euler_numerics.cuh"
using namespace eu;
// in: 6 floats per problem (rL, uL, pL, rR, uR, pR); out: 6 doubles
// (p, u, ok) of the mixed route and of the FP64 iteration
__global__ void k(const float* in, double* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* s = in + 6 * (size_t)i;
    const float aL = sqrtf(1.4f * s[2] / s[0]), aR = sqrtf(1.4f * s[5] / s[3]);
    const StarD m = exact_star_mixed(s[0], s[1], s[2], aL, s[3], s[4], s[5], aR);
    const PrimD L{(double)s[0], (double)s[1], 0.0, (double)s[2], (double)aL};
    const PrimD R{(double)s[3], (double)s[4], 0.0, (double)s[5], (double)aR};
    double p = 0.0, u = 0.0;
    const bool ok = exact_star(L, R, p, u);
    double* o = out + 6 * (size_t)i;
    o[0] = m.p; o[1] = m.u; o[2] = m.ok ? 1.0 : 0.0;
    o[3] = p; o[4] = u; o[5] = ok ? 1.0 : 0.0;
}
int main(int argc, char** argv) {
    FILE* f = fopen(argv[1], "rb");
    int n = 0;
    if (!f || fread(&n, sizeof(int), 1, f) != 1 || n <= 0) return 2;
    float* h = new float[6 * (size_t)n];
    if (fread(h, sizeof(float), 6 * (size_t)n, f) != 6 * (size_t)n) return 2;
    fclose(f);
    float* din;
    double* dout;
    if (cudaMalloc(&din, 6 * sizeof(float) * (size_t)n) != cudaSuccess) return 3;
    if (cudaMalloc(&dout, 6 * sizeof(double) * (size_t)n) != cudaSuccess) return 3;
    cudaMemcpy(din, h, 6 * sizeof(float) * (size_t)n, cudaMemcpyHostToDevice);
    k<<<(n + 255) / 256, 256>>>(din, dout, n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    double* o = new double[6 * (size_t)n];
    cudaMemcpy(o, dout, 6 * sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost);
    f = fopen(argv[2], "wb");
    fwrite(o, sizeof(double), 6 * (size_t)n, f);
    fclose(f);
    return 0;
}
"""


def problems(rng, n):
    """Random face states (FP32): densities 1e-3..1e3, pressures 1e-4..1e2,
    velocities up to +-6 (vacuum generation included), plus hand-picked
    families."""
    r = 10.0 ** rng.uniform(-3, 3, (n, 2))
    p = 10.0 ** rng.uniform(-4, 2, (n, 2))
    u = rng.uniform(-6, 6, (n, 2))
    P = np.stack([r[:, 0], u[:, 0], p[:, 0], r[:, 1], u[:, 1], p[:, 1]], axis=1)
    fam = [
        [1.0, 0.0, 1.0, 0.125, 0.0, 0.1],          # Sod
        [1.0, 0.0, 1000.0, 1.0, 0.0, 0.01],        # strong blast (ratio 1e5)
        [1.0, -2.0, 0.4, 1.0, 2.0, 0.4],           # 123 problem (strong rarefactions)
        [1.0, -20.0, 0.4, 1.0, 20.0, 0.4],         # vacuum generation
        [5.99924, 19.5975, 460.894, 5.99242, -6.19633, 46.095],   # colliding shocks
        [1.0, 0.0, 1.0, 1.0, 0.0, 1.0 + 1e-6],     # nearly equal pressures
        [1.0, 0.0, 1.0, 2.0, 0.0, 1.0],            # contact only (p* = p)
        [1.0, 0.5, 1.0, 1.0, 0.5, 1.0],            # identical states
        [1e-3, 0.0, 1e-4, 1e3, 0.0, 1e2],          # extreme density / pressure ratios
    ]
    return np.concatenate([P, np.asarray(fam)]).astype(np.float32)


def test_mixed_route_matches_fp64_iteration(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "mixed.cu"
    src.write_text(SRC)
    exe = tmp_path / "mixed"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", f"-I{CSRC}",
                    "-o", str(exe), str(src)], check=True)
    rng = np.random.default_rng(11)
    P = problems(rng, 1 << 18)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(np.int32(len(P)).tobytes())
        f.write(P.tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([str(exe), str(inp), str(out)], check=True)
    o = np.fromfile(out, dtype=np.float64).reshape(-1, 6)
    pm, um, okm, pd, ud, okd = o.T
    assert np.array_equal(okm, okd)
    ok = okd == 1.0
    a = np.sqrt(1.4 * P[:, [2, 5]].astype(np.float64) / P[:, [0, 3]].astype(np.float64)).max(axis=1)
    # converged FP64 iterations: |dp| < 1e-8 mean at the last step, so its p*
    # is exact to ~1e-15; the mixed route lands within 1e-10
    conv = ok & (pd > 1e-11)
    rel_p = np.abs(pm[conv] - pd[conv]) / pd[conv]
    rel_u = np.abs(um[conv] - ud[conv]) / (np.abs(ud[conv]) + a[conv])
    print(f"max rel p* {rel_p.max():.2e}, max rel u* {rel_u.max():.2e}, "
          f"{conv.sum()} converged of {len(P)}")
    assert rel_p.max() <= 1e-10, rel_p.max()
    assert rel_u.max() <= 1e-10, rel_u.max()
    # p* at or below 1e-11: vacuum generation, where the FP64 iteration
    # halves toward p = 0 and the mixed route returns its bits, or a
    # near-vacuum root that both find
    tiny = ok & ~conv
    same = (pm[tiny] == pd[tiny]) & (um[tiny] == ud[tiny])
    close = (np.abs(pm[tiny] - pd[tiny]) <= 1e-10 * np.maximum(pd[tiny], 1e-12)) & \
            (np.abs(um[tiny] - ud[tiny]) <= 1e-10 * (np.abs(ud[tiny]) + a[tiny]))
    assert np.all(same | close)
    vac = len(P) - 6                       # the hand-picked vacuum-generating problem
    assert tiny[vac] and pm[vac] == pd[vac] and um[vac] == ud[vac]
