"""The FP64-free barycentric fast path of the CUDA kernels (fr_exact.cuh),
compiled for the host, against the reference's literal double arithmetic on
random triangles of every size class, including edge lattice points."""

import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fast_barycentric_is_bit_exact(tmp_path):
    exe = str(tmp_path / "test_exact")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    f"-I{ROOT}/forkerrenderer_gb300/csrc", f"{ROOT}/tests/cpp/test_exact.cpp",
                    "-o", exe], check=True)
    for seed in ("1", "2", "3"):
        r = subprocess.run([exe, "200000", seed], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "mismatches 0" in r.stdout


def test_ssao_estimate_bound_holds(tmp_path):
    """The SSAO estimate's error bound (fr_ssao.cuh), compiled for the host: the
    exact viewport x, y, z of every sample lies inside the estimate's test
    interval, on random cameras, points and offsets, with the estimate's
    approximate reciprocal pushed 2 ulp either way."""
    exe = str(tmp_path / "test_ssao")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    f"-I{ROOT}/forkerrenderer_gb300/csrc", f"{ROOT}/tests/cpp/test_ssao.cpp",
                    "-o", exe], check=True)
    for seed in ("1", "2", "3"):
        r = subprocess.run([exe, "100000", seed], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "outside the interval 0;" in r.stdout
