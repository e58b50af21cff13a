"""The C++ drop-in (include/ts_kernel.hpp: GpuExplicitRungeKuttaFVM, a
subclass of the reference's Kernel, and CreateGpuKernel) compiled against the
reference's own headers and linked with libtsfvm.so, where the reference
checkout exists (oracle/ref_build/Makefile, target `dropin`).  The check
program sets up a Sod tube and a 2D channel whose bottom side is
position-dependent (DomainBCinfo::isComplex with getMarker) the way the
reference's drivers do; here it prints the ts_config the subclass builds,
which must be the library's own description of the same problems."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

REF = "/root/reference"
pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")),
                                reason="the reference checkout is not on this host")


@pytest.fixture(scope="module")
def dropin(tslib):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref_build"), "REF=" + REF, "dropin"],
                   check=True)
    return os.path.join(ROOT, "oracle", "_ref", "gpu_dropin")


def parse(out):
    lines = {}
    for ln in out.splitlines():
        w = ln.split()
        if len(w) > 2 and w[0] in ("sod1d", "plate2d"):
            lines.setdefault(w[0], []).append(w[1:])
    return lines


def test_dropin_builds_the_same_configuration(dropin, tmp_path):
    from turbostructred_gb300 import capi
    r = subprocess.run([dropin, "--config"], cwd=tmp_path, capture_output=True, text=True, check=True)
    cfg = parse(r.stdout)
    def fields(tokens):
        return {k: tokens[i + 1] for i, k in enumerate(tokens[:-1]) if not k.replace(".", "").lstrip("-").isdigit()}

    head = fields(cfg["plate2d"][0])
    assert head["n_dims"] == "2" and head["nx"] == "64" and head["ny"] == "32"
    assert head["recon"] == str(capi.RECON_LINEAR2_LIM) and head["solver"] == str(capi.RS_ROE)
    assert float(head["eps"]) == 0.05 and float(head["cfl"]) == 0.45
    assert head["precision"] == str(capi.PRECISION_MIXED) and head["residual_norms"] == "1"
    sides = {int(w[1]): w for w in cfg["plate2d"] if w[0] == "side"}
    assert int(sides[0][3]) == capi.BC_SUBSONIC_INLET and float(sides[0][5]) == 1.0
    kinds = [int(w[3]) for w in cfg["plate2d"] if w[0] == "kind"]
    assert kinds == [capi.BC_SYMMETRY, capi.BC_WALL]
    marks = np.array([int(x) for x in sides[2][sides[2].index("markers") + 1:]])
    # the same split described to the library: kinds 0 (Symmetry) below x = 0.3, 1 (Wall) above
    case = capi.make_case(ndims=2, nx=64, ny=32, length=(1.0, 0.5, 1.0), periodic=(0, 0, 1),
                          bc_kinds=[(capi.BC_SYMMETRY, 0.0, (0, 0, 0), 0.0), (capi.BC_WALL, 0.0, (0, 0, 0), 0.0)],
                          bc_split={2: (0, 0.3, 0, 1)})
    assert np.array_equal(marks, capi.split_markers(case)[2])
    sod = fields(cfg["sod1d"][0])
    assert sod["nx"] == "200" and float(sod["save_solution_time"]) == 0.05 and sod["recon"] == "0"


def test_dropin_reaches_the_library(dropin, tmp_path):
    """Init, SetInitialConditions and Run go through the subclass into
    ts_create; without a GPU the library reports that, with one the check
    program compares the GPU results with the reference's CPU kernel."""
    import torch
    r = subprocess.run([dropin], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stdout[-2000:]
    else:
        assert r.returncode == 3
        assert "no CUDA device available" in r.stdout
