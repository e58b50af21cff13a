"""Solution files in the reference's formats (include/ts_fvm.h, solution files).

The reference's own Kernel::SaveSolution, LoadSolution and
SaveSolutionToTecplot outputs (tests/golden/io, made by make_io_golden.py
from the reference's code) are the bar, byte for byte:
  * host writers: the fixture's final state -> the same .bin and .dat bytes;
  * host reader: the fixture's .bin -> the same state and time;
  * device (FP64 path, bit-for-bit with the reference): the same initial
    state stepped the same number of times -> the same file bytes from
    ts_save_solution / ts_save_tecplot (synchronous and asynchronous), and
    ts_load_solution of a reference file followed by more steps -> the
    reference's state and time after its own LoadSolution.
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT

IO = os.path.join(ROOT, "tests", "golden", "io")
NAMES = ["io_sod1d", "io_quad2d", "io_blast3d"]


def load(name):
    d = dict(np.load(os.path.join(IO, name + ".npz")))
    meta = json.loads(bytes(d.pop("meta")).decode())
    case = meta["case"]
    case["periodic"] = tuple(case["periodic"])
    case["length"] = tuple(case["length"])
    case["bc"] = [(t, dens, tuple(vel), ps) for t, dens, vel, ps in case["bc"]]
    case["blocks"] = {}
    d["case"], d["meta"] = case, meta
    d["iteration"], d["time"] = int(d["scalars"][0]), float(d["scalars"][1])
    return d


def blob(name, ext):
    with open(os.path.join(IO, name + ext), "rb") as f:
        return f.read()


@pytest.mark.parametrize("name", NAMES)
def test_host_writers_match_reference_bytes(name, tslib, tmp_path):
    from turbostructred_gb300 import capi
    g = load(name)
    case = capi.make_case(**g["case"])
    state = g["final"].reshape(capi.interior_shape(case))
    capi.write_solution_file(case, state, g["time"], str(tmp_path / "s.bin"))
    assert (tmp_path / "s.bin").read_bytes() == blob(name, ".bin")
    capi.write_tecplot_file(case, state, g["time"], str(tmp_path / "s.dat"), g["meta"]["molar_mass"],
                            g["meta"]["gas_constant"])
    assert (tmp_path / "s.dat").read_bytes() == blob(name, ".dat")


@pytest.mark.parametrize("name", NAMES)
def test_host_reader_matches_reference_file(name, tslib):
    from turbostructred_gb300 import capi
    g = load(name)
    case = capi.make_case(**g["case"])
    values, t = capi.read_solution_file(case, os.path.join(IO, name + ".bin"))
    assert t == g["time"]
    assert np.array_equal(values, g["final"].reshape(values.shape))


def test_reader_refuses_other_ranks_and_short_files(tslib, tmp_path):
    from turbostructred_gb300 import capi
    g = load("io_sod1d")
    case = capi.make_case(**g["case"])
    b = bytearray(blob("io_sod1d", ".bin"))
    b[8:12] = (3).to_bytes(4, "little")
    (tmp_path / "r3.bin").write_bytes(bytes(b))
    with pytest.raises(capi.TsError) as e:
        capi.read_solution_file(case, str(tmp_path / "r3.bin"))
    assert e.value.status == 2
    (tmp_path / "short.bin").write_bytes(blob("io_sod1d", ".bin")[:100])
    with pytest.raises(capi.TsError) as e:
        capi.read_solution_file(case, str(tmp_path / "short.bin"))
    assert e.value.status == 1


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_device_save_matches_reference_bytes(name, tslib, tmp_path):
    from turbostructred_gb300 import capi
    g = load(name)
    case = capi.make_case(**g["case"])
    with capi.Solver(case, precision=capi.PRECISION_FP64) as s:
        s.set_state(g["initial"])
        info = s.step(g["meta"]["steps"])
        assert info["iteration"] == g["iteration"] and info["time"] == g["time"]
        s.save_solution(str(tmp_path / "s.bin"))
        mm, rg = g["meta"]["molar_mass"], g["meta"]["gas_constant"]
        s.save_tecplot(str(tmp_path / "s.dat"), mm, rg)
        s.save_tecplot(str(tmp_path / "a.dat"), mm, rg, asynchronous=True)
        s.step(2)  # the asynchronous write holds its own snapshot
        s.wait_writes()
    assert (tmp_path / "s.bin").read_bytes() == blob(name, ".bin")
    assert (tmp_path / "s.dat").read_bytes() == blob(name, ".dat")
    assert (tmp_path / "a.dat").read_bytes() == blob(name, ".dat")


@pytest.mark.gpu
def test_device_load_matches_reference_restart(tslib, tmp_path):
    from turbostructred_gb300 import capi
    g = load("io_load2d")
    case = capi.make_case(**g["case"])
    with capi.Solver(case, precision=capi.PRECISION_FP64) as s:
        s.set_state(np.ones(capi.interior_shape(case)))
        s.load_solution(os.path.join(IO, "io_quad2d.bin"))
        info = s.info()
        assert info["time"] == load("io_quad2d")["time"] and info["iteration"] == 0
        assert info["next_solution_time"] == 0.02
        info = s.step(4)
        got = s.get_state()
        s.save_solution(str(tmp_path / "l.bin"))
    assert info["time"] == g["time"]
    assert np.array_equal(got, g["final"].reshape(got.shape))
    assert (tmp_path / "l.bin").read_bytes() == blob("io_load2d", ".bin")
