"""pow_third (csrc/ocpx_common.cuh), the cube root the flash uses in place of
pow(x, 1.0/3), against a long-double evaluation of x^fl(1/3) and against
CUDA's own pow: within 2 ulp of the former, like CUDA's pow."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "opencaeporox_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "ocpx_common.cuh"
__global__ void k(const double* x, double* a, double* b, int n)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) { a[t] = ocpx::pow_third(x[t]); b[t] = pow(x[t], 1.0 / 3); }
}
int main(int argc, char** argv)
{
    FILE* f = fopen(argv[1], "rb");
    int n = 0;
    if (fread(&n, sizeof(int), 1, f) != 1) return 2;
    std::vector<double> x(n), a(n), b(n);
    if (fread(x.data(), sizeof(double), n, f) != (size_t)n) return 2;
    fclose(f);
    double *dx, *da, *db;
    cudaMalloc(&dx, n * 8); cudaMalloc(&da, n * 8); cudaMalloc(&db, n * 8);
    cudaMemcpy(dx, x.data(), n * 8, cudaMemcpyHostToDevice);
    k<<<(n + 255) / 256, 256>>>(dx, da, db, n);
    cudaMemcpy(a.data(), da, n * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), db, n * 8, cudaMemcpyDeviceToHost);
    if (cudaDeviceSynchronize() != cudaSuccess) return 3;
    f = fopen(argv[2], "wb");
    fwrite(a.data(), 8, n, f); fwrite(b.data(), 8, n, f);
    fclose(f);
    return 0;
}
"""


def ulp_err(got, ref_ld):
    ref = ref_ld.astype(np.float64)
    spacing = np.spacing(np.abs(ref))
    return np.abs((got.astype(np.longdouble) - ref_ld) / spacing.astype(np.longdouble)).astype(np.float64)


def test_pow_third_accuracy(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "p.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "p"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-I", CSRC, str(src), "-o", str(exe)], check=True)
    rng = np.random.default_rng(7)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 200000), rng.uniform(0, 10, 50000),
                        np.ldexp(1.0, np.arange(-1070, 1020)), [5e-324, 1.0, 8.0, 27.0, 0.125]])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(np.int32(x.size).tobytes())
        f.write(x.astype(np.float64).tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([str(exe), str(inp), str(out)], check=True)
    r = np.fromfile(out, dtype=np.float64)
    mine, cuda = r[: x.size], r[x.size:]
    ref = np.power(x.astype(np.longdouble), np.longdouble(1.0 / 3))
    ok = x > 1e-300  # long double covers the full double range on both hosts; skip extreme subnormals
    e_mine = ulp_err(mine[ok], ref[ok])
    e_cuda = ulp_err(cuda[ok], ref[ok])
    assert np.max(e_mine) <= 2.0, np.max(e_mine)
    assert np.max(e_mine) <= max(np.max(e_cuda), 1.0) + 1.0
    assert np.all(np.isfinite(mine))
