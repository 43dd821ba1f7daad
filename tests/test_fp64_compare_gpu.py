"""The FP64 comparisons that run on the integer pipes (Ar<double>::gt,
finite, fmin_, fmax_, minmod<double> and physical_recon<double> in
large_sys_eq_opt_gb300/csrc/euler_numerics.cuh) against IEEE comparisons in
numpy, on special values (signed zeros, infinities, NaNs of both signs,
subnormals, the 1e-14 and 1e-12 thresholds) and random bit patterns: the
same booleans everywhere, fmin/fmax values equal (the non-NaN argument for
one NaN, as CUDA's fmin/fmax), and minmod equal to max(0, min(a, b)) + min(0, max(a, b))."""
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
using A = Ar<double>;
// per pair (x, y): finite(x), gt(x, c) for 5 thresholds c, the recon
// physicality test of (rho, u_n, u_t, p) = (x, y, 1, x) and of (1, 1, y, x)
// (8 flags as doubles), then fmin, fmax, minmod
__global__ void k(const double* xy, double* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = xy[2 * (size_t)i], y = xy[2 * (size_t)i + 1];
    const double cs[5] = {0.0, 1.0e-14, 1.0e-12, 4.0e-12, 1.0};
    double* o = out + 17 * (size_t)i;
    o[0] = A::finite(x);
    for (int c = 0; c < 5; ++c) o[1 + c] = A::gt(x, cs[c]);
    o[6] = physical_recon(Prim<double>{x, y, 1.0, x, 0.0});
    o[7] = physical_recon(Prim<double>{1.0, 1.0, y, x, 0.0});
    for (int c = 8; c < 14; ++c) o[c] = 0.0;
    o[14] = A::fmin_(x, y); o[15] = A::fmax_(x, y); o[16] = minmod<double>(x, y);
}
int main(int argc, char** argv) {
    FILE* f = fopen(argv[1], "rb");
    int n = 0;
    if (!f || fread(&n, sizeof(int), 1, f) != 1 || n <= 0) return 2;
    double* h = new double[2 * (size_t)n];
    if (fread(h, sizeof(double), 2 * (size_t)n, f) != 2 * (size_t)n) return 2;
    fclose(f);
    double *din, *dout;
    if (cudaMalloc(&din, 2 * sizeof(double) * (size_t)n) != cudaSuccess) return 3;
    if (cudaMalloc(&dout, 17 * sizeof(double) * (size_t)n) != cudaSuccess) return 3;
    cudaMemcpy(din, h, 2 * sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
    k<<<(n + 255) / 256, 256>>>(din, dout, n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    double* o = new double[17 * (size_t)n];
    cudaMemcpy(o, dout, 17 * sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost);
    f = fopen(argv[2], "wb");
    fwrite(o, sizeof(double), 17 * (size_t)n, f);
    fclose(f);
    return 0;
}
"""


def values(rng):
    special = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, -np.nan, 5e-324, -5e-324,
                        1e-14, -1e-14, np.nextafter(1e-14, 1), np.nextafter(1e-14, 0), 1e-12, 4e-12,
                        2e-12, 1e308, -1e308, 0.5, -0.5, 3.0, -3.0])
    nan_payload = np.array([0x7ff8000000000001, 0xfff0000000000001], dtype=np.uint64).view(np.float64)
    sign = rng.integers(0, 2, 20000, dtype=np.int64) << np.int64(63)
    rand_bits = (rng.integers(0, 2**63, 20000, dtype=np.int64) | sign).view(np.float64)
    rand_vals = rng.uniform(-5, 5, 20000)
    v = np.concatenate([special, nan_payload, rand_bits, rand_vals])
    x = np.repeat(special, len(special))
    y = np.tile(special, len(special))
    xr = rng.permutation(v)
    yr = rng.permutation(v)
    return np.concatenate([x, xr]), np.concatenate([y, yr])


def test_integer_pipe_comparisons_match_ieee(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "cmp.cu"
    src.write_text(SRC)
    exe = tmp_path / "cmp"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", f"-I{CSRC}",
                    "-o", str(exe), str(src)], check=True)
    x, y = values(np.random.default_rng(5))
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(np.int32(len(x)).tobytes())
        f.write(np.stack([x, y], axis=1).astype(np.float64).tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([str(exe), str(inp), str(out)], check=True)
    o = np.fromfile(out, dtype=np.float64).reshape(-1, 17)
    with np.errstate(invalid="ignore", over="ignore"):
        assert np.array_equal(o[:, 0] == 1, np.isfinite(x))
        for c, cv in enumerate((0.0, 1e-14, 1e-12, 4e-12, 1.0)):
            assert np.array_equal(o[:, 1 + c] == 1, x > cv), cv
        # physical_recon (src/cpu/solver_cpu.cpp:39-43): finite velocities,
        # 1e-12 < rho, p < inf
        rec = np.isfinite(y) & (x > 1e-12) & (x < np.inf)
        assert np.array_equal(o[:, 6] == 1, rec)
        assert np.array_equal(o[:, 7] == 1, rec)
        # fmin / fmax: the non-NaN argument for one NaN (quiet or signalling,
        # as CUDA's fmin/fmax), NaN for two.  Written out, since numpy's fmin
        # on Arm returns NaN for a signalling NaN.
        for col, op in ((14, np.minimum), (15, np.maximum)):
            ref = np.where(np.isnan(y), x, np.where(np.isnan(x), y, op(x, y)))
            assert np.array_equal(o[:, col], ref, equal_nan=True), col
        # minmod (non-NaN pairs): the value of max(0, min) + min(0, max)
        ok = ~np.isnan(x) & ~np.isnan(y) & ~(np.isinf(x) & np.isinf(y))
        ref = np.maximum(0.0, np.minimum(x, y)) + np.minimum(0.0, np.maximum(x, y))
        assert np.array_equal(o[ok, 16], ref[ok])
