"""The FP64 reciprocal seventh root of the exact solver (rroot7 in
large_sys_eq_opt_gb300/csrc/euler_numerics.cuh: Newton's iteration seeded
with the FP32 power) against CUDA's pow(r, -1/7): at most a few ulp over
pressure ratios from 1e-30 to 1e30, and pow's own results outside that range
and for 0, infinity and NaN."""
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
#include <cstring>
#include <cuda_runtime.h>
#include "euler_numerics.cuh"
__global__ void k(const double* r, double* w, double* ref, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    w[i] = eu::rroot7<double>(r[i]);
    ref[i] = pow(r[i], -1.0 / 7.0);
}
int main(int argc, char** argv) {
    FILE* f = fopen(argv[1], "rb");
    int n = 0;
    if (!f || fread(&n, sizeof(int), 1, f) != 1 || n <= 0) return 2;
    double* h = new double[3 * (size_t)n];
    if (fread(h, sizeof(double), n, f) != (size_t)n) return 2;
    fclose(f);
    double* d;
    if (cudaMalloc(&d, 3 * sizeof(double) * (size_t)n) != cudaSuccess) return 3;
    cudaMemcpy(d, h, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
    k<<<(n + 255) / 256, 256>>>(d, d + n, d + 2 * (size_t)n, n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    cudaMemcpy(h + n, d + n, 2 * sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost);
    f = fopen(argv[2], "wb");
    fwrite(h + n, sizeof(double), 2 * (size_t)n, f);
    fclose(f);
    return 0;
}
"""


def test_rroot7_matches_pow(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "rroot7.cu"
    src.write_text(SRC)
    exe = tmp_path / "rroot7"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", f"-I{CSRC}",
                    "-o", str(exe), str(src)], check=True)
    rng = np.random.default_rng(7)
    r = np.concatenate([10.0 ** rng.uniform(-30.0, 30.0, 1 << 20),      # the Newton range
                        10.0 ** rng.uniform(-300.0, -30.5, 4096),       # pow() outside it
                        10.0 ** rng.uniform(30.5, 300.0, 4096),
                        [1.0, 1.0e-30, 1.0e30, 0.0, np.inf, np.nan, 5e-324]])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(np.int32(len(r)).tobytes())
        f.write(r.astype(np.float64).tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([str(exe), str(inp), str(out)], check=True)
    res = np.fromfile(out, dtype=np.float64).reshape(2, -1)
    w, ref = res[0], res[1]
    fin = np.isfinite(ref) & (ref > 0)
    ulp = np.abs(w[fin].view(np.int64) - ref[fin].view(np.int64))
    assert int(ulp.max()) <= 8, int(ulp.max())
    assert np.array_equal(np.isnan(w), np.isnan(ref))
    assert np.array_equal(w[~fin & ~np.isnan(ref)], ref[~fin & ~np.isnan(ref)])
    # outside [1e-30, 1e30] the result is pow's own
    outside = (r < 1e-30) | (r > 1e30)
    assert np.array_equal(w[outside & fin], ref[outside & fin])
