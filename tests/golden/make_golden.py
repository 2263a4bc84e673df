"""Regenerate the golden fixtures in this directory (run in a checkout that has the MPPI-Generic sources).

* reference_kats.npz — inputs and known answers of the reference's normexp and weighted-reduction kernel tests,
  produced by gen_reference_kats.cpp with the tests' own std::default_random_engine(7) recipes.
* tsallis_kats.npz — the reference's TsallisTransform compiled for the host and run on seeded costs.
* colored_noise.npz — the reference's NumPy colored-noise generator (scripts/colored_noise.py,
  powerlaw_psd_gaussian) run with injected standard normals for the real and imaginary spectrum parts, so the
  engine's colored-noise shaping can be compared against it given the same normals.

Usage: python tests/golden/make_golden.py /path/to/mppi_generic_vendor
"""
from __future__ import annotations

import importlib.util
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def reference_kats():
    with tempfile.TemporaryDirectory() as td:
        exe = Path(td) / "gen"
        subprocess.run(["g++", "-O0", "-std=c++17", "-o", str(exe), str(HERE / "gen_reference_kats.cpp")], check=True)
        subprocess.run([str(exe), td], check=True)
        rd = lambda n, dt: np.fromfile(Path(td) / n, dtype=dt)  # noqa: E731
        np.savez_compressed(
            HERE / "reference_kats.npz",
            baseline_costs=rd("baseline_costs.f32", np.float32), baseline_known=rd("baseline_known.f32", np.float32),
            normalizer_costs=rd("normalizer_costs.f32", np.float32),
            normalizer_known=rd("normalizer_known.f32", np.float32),
            expnorm_costs=rd("expnorm_costs.f32", np.float32), expnorm_known=rd("expnorm_known.f32", np.float32),
            wr_weights=rd("wr_weights.f32", np.float32), wr_controls=rd("wr_controls.f32", np.float32),
            wr_normalizer=rd("wr_normalizer.f32", np.float32), wr_known=rd("wr_known.f64", np.float64))


def colored_noise(ref_root: Path):
    spec = importlib.util.spec_from_file_location("ref_colored_noise", ref_root / "scripts" / "colored_noise.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    rng = np.random.default_rng(20240511)
    out = {}
    for case, (T, beta, fmin, batch) in enumerate([(32, 1.0, 0.0, 8), (64, 1.0, 0.0, 8), (128, 2.0, 0.0, 4),
                                                     (50, 0.5, 0.0, 6), (64, 1.0, 0.05, 4), (33, 1.0, 0.0, 4)]):
        N = 2 * T
        F = N // 2 + 1
        zr = rng.standard_normal((batch, F)).astype(np.float32)
        zi = rng.standard_normal((batch, F)).astype(np.float32)
        draws = [zr, zi]

        def normal(scale=1.0, size=None):
            z = draws.pop(0).astype(np.float64)
            return z * scale

        mod.normal = normal
        y = mod.powerlaw_psd_gaussian(beta, (batch, N), fmin=fmin)
        out[f"c{case}_T"] = np.int32(T)
        out[f"c{case}_beta"] = np.float32(beta)
        out[f"c{case}_fmin"] = np.float32(fmin)
        out[f"c{case}_zr"] = zr
        out[f"c{case}_zi"] = zi
        out[f"c{case}_y"] = y.astype(np.float64)
    np.savez_compressed(HERE / "colored_noise.npz", **out)


TSALLIS_CASES = [(5.0, 2.0), (20.0, 1.5), (2.5, 3.0), (0.7, 1.25)]


def tsallis_kats(ref_root: Path):
    """tsallis_kats.npz: the reference's own TsallisTransform (include/mppi/core/mppi_common.cu:1004-1021, a
    __device__ __host__ function with no dependencies) compiled for the host from the checkout at generation time and
    run on seeded cost vectors.  Only its outputs are stored; the function's text is read from the checkout into a
    temporary directory and never kept."""
    src = (ref_root / "include" / "mppi" / "core" / "mppi_common.cu").read_text()
    start = src.index("__device__ __host__ inline void TsallisTransform(")
    body = src.index("{", start)
    depth, end = 0, body
    for end in range(body, len(src)):
        depth += {"{": 1, "}": -1}.get(src[end], 0)
        if depth == 0:
            break
    func = src[start:end + 1]
    driver = """#include <cmath>
#include <cstdio>
#include <vector>
#define __device__
#define __host__
#define __restrict__
%s
int main(int argc, char** argv)
{
  float gamma, r, baseline; int n;
  if (fread(&gamma, 4, 1, stdin) != 1 || fread(&r, 4, 1, stdin) != 1 || fread(&baseline, 4, 1, stdin) != 1 ||
      fread(&n, 4, 1, stdin) != 1) return 1;
  std::vector<float> c(n);
  if (fread(c.data(), 4, n, stdin) != (size_t)n) return 1;
  TsallisTransform(n, c.data(), gamma, r, baseline, 0, 1);
  fwrite(c.data(), 4, n, stdout);
  return 0;
}
""" % func
    rng = np.random.default_rng(20241204)
    out = {}
    with tempfile.TemporaryDirectory() as td:
        cpp, exe = Path(td) / "tsallis.cpp", Path(td) / "tsallis"
        cpp.write_text(driver)
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", str(exe), str(cpp)], check=True)
        for i, (gamma, r) in enumerate(TSALLIS_CASES):
            c = (100.0 + rng.exponential(gamma / 2, 4096)).astype(np.float32)
            b = np.float32(c.min())
            payload = (np.array([gamma, r, b], np.float32).tobytes() + np.array([c.size], np.int32).tobytes()
                       + c.tobytes())
            res = subprocess.run([str(exe)], input=payload, capture_output=True, check=True)
            out[f"t{i}_gamma"] = np.float32(gamma)
            out[f"t{i}_r"] = np.float32(r)
            out[f"t{i}_baseline"] = b
            out[f"t{i}_costs"] = c
            out[f"t{i}_weights"] = np.frombuffer(res.stdout, np.float32).copy()
    np.savez_compressed(HERE / "tsallis_kats.npz", **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the MPPI-Generic checkout>")
    ref = Path(sys.argv[1])
    reference_kats()
    colored_noise(ref)
    tsallis_kats(ref)
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))
