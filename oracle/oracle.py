"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracle.

``fvm_oracle.c`` restates the reference solver's explicit FVM step
(TurboStructred ``src/Methods/ExplicitRungeKuttaFVM.h``) in C and is the parity
checker for the CUDA path.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU legs use this module; the product package never imports it.

Problems are described by a plain ``dict`` (see :func:`make_case`) that the
tests also hand to the product's C-ABI, so both sides see the same setup.

``run_reference`` drives the reference's own code (``oracle/_ref/ref_run``,
built by ``oracle/ref_build/Makefile`` from the reference sources) and is used
only where those sources exist, to generate the committed golden fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_RUN = os.path.join(HERE, "_ref", "ref_run")

MAX_BLOCKS = 16
MAX_BC_KINDS = 8
BC_IDS = 6 + MAX_BC_KINDS

# Enum values: MethodConfiguration.h:5-23, BoundaryConditionConfiguration.h:12-19
RECON_PWC, RECON_LINEAR2, RECON_ENO2, RECON_LINEAR2_LIM = 0, 1, 2, 3
LIM_BJ, LIM_VENKAT = 0, 1
RS_GODUNOV, RS_ROE, RS_NONE, RS_HLLC = 0, 1, 2, 3
BC_WALL, BC_SYMMETRY, BC_MOVING_WALL, BC_SUBSONIC_INLET, BC_SUBSONIC_OUTLET, BC_NATURAL = range(6)
EOS_IDEAL, EOS_STIFFENED = 0, 1


class OrcConfig(C.Structure):
    _fields_ = [
        ("ndims", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("periodic", C.c_int * 3),
        ("length", C.c_double * 3),
        ("n_blocks", C.c_int * 3),
        ("block_pos", (C.c_double * MAX_BLOCKS) * 3),
        ("block_q", (C.c_double * MAX_BLOCKS) * 3),
        ("block_cells", (C.c_int * MAX_BLOCKS) * 3),
        ("gamma", C.c_double), ("eos", C.c_int), ("p_inf", C.c_double),
        ("recon", C.c_int), ("limiter", C.c_int), ("solver", C.c_int),
        ("eps", C.c_double), ("cfl", C.c_double),
        ("max_iteration", C.c_int),
        ("max_time", C.c_double), ("save_solution_time", C.c_double), ("save_slice_time", C.c_double),
        ("bc_type", C.c_int * BC_IDS),
        ("bc_density", C.c_double * BC_IDS),
        ("bc_velocity", (C.c_double * 3) * BC_IDS),
        ("bc_pstatic", C.c_double * BC_IDS),
        ("threads", C.c_int),
        ("external_force", C.c_int), ("uniform_acceleration", C.c_int),
        ("sigma", C.c_double * 3), ("acceleration", C.c_double * 3),
        ("viscous", C.c_int), ("viscosity", C.c_double),
        ("bc_marker", C.POINTER(C.c_ubyte) * 6),
    ]


class OrcStepInfo(C.Structure):
    _fields_ = [
        ("iteration", C.c_int), ("time", C.c_double), ("dt", C.c_double),
        ("next_solution_time", C.c_double), ("next_slice_time", C.c_double),
        ("residual", C.c_double * 5),
    ]


def build_oracle(force: bool = False) -> str:
    """Compile fvm_oracle.c into oracle/liboracle.so (OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "fvm_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src),
                                                 os.path.getmtime(os.path.join(HERE, "fvm_oracle.h")))):
        return LIB_PATH
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
           "-shared", src, "-o", LIB_PATH + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(LIB_PATH)
        L.orc_advance.argtypes = [C.POINTER(OrcConfig), C.POINTER(C.c_double), C.c_int, C.POINTER(OrcStepInfo)]
        L.orc_advance.restype = C.c_int
        L.orc_grid.argtypes = [C.POINTER(OrcConfig)] + [C.POINTER(C.c_double)] * 6
        L.orc_exact_riemann.argtypes = [C.c_double] * 9 + [C.POINTER(C.c_double)] * 3
        L.orc_exact_riemann.restype = C.c_int
        L.orc_fill_scenario.argtypes = [C.POINTER(OrcConfig), C.c_int, C.c_ulonglong, C.POINTER(C.c_double), C.c_int,
                                        C.POINTER(C.c_double)]
        L.orc_fill_scenario.restype = C.c_int
        L.orc_hash_uniform.argtypes = [C.c_ulonglong, C.c_longlong, C.c_longlong, C.c_longlong]
        L.orc_hash_uniform.restype = C.c_double
        _lib = L
    return _lib


def make_case(**kw) -> dict:
    """A problem description shared by the oracle, the reference driver and the
    product's C-ABI.  Defaults follow KernelConfiguration.h:21-93."""
    case = dict(ndims=1, nx=1, ny=1, nz=1, periodic=(1, 1, 1), length=(1.0, 1.0, 1.0), blocks={},
                gamma=1.4, eos=EOS_IDEAL, p_inf=0.0, recon=RECON_PWC, limiter=LIM_BJ, solver=RS_ROE,
                eps=0.0, cfl=0.25, max_iter=1000, max_time=1.0, save_solution_time=0.0,
                save_slice_time=0.0, bc=[(BC_NATURAL, 0.0, (0.0, 0.0, 0.0), 0.0)] * 6,
                external_force=None, uniform_acceleration=None, viscous=False, viscosity=0.0,
                bc_kinds=[], bc_split={})
    case.update(kw)
    return case


def to_struct(case: dict, threads: int = 0) -> OrcConfig:
    c = OrcConfig()
    c.ndims, c.nx, c.ny, c.nz = case["ndims"], case["nx"], case["ny"], case["nz"]
    for a in range(3):
        c.periodic[a] = int(case["periodic"][a])
        c.length[a] = case["length"][a]
        blocks = case["blocks"].get(a, []) if isinstance(case["blocks"], dict) else []
        c.n_blocks[a] = len(blocks)
        for b, (pos, q, n) in enumerate(blocks):
            c.block_pos[a][b], c.block_q[a][b], c.block_cells[a][b] = pos, q, n
    c.gamma, c.eos, c.p_inf = case["gamma"], case["eos"], case["p_inf"]
    c.recon, c.limiter, c.solver = case["recon"], case["limiter"], case["solver"]
    c.eps, c.cfl = case["eps"], case["cfl"]
    c.max_iteration, c.max_time = case["max_iter"], case["max_time"]
    c.save_solution_time, c.save_slice_time = case["save_solution_time"], case["save_slice_time"]
    for s, (t, dens, vel, ps) in enumerate(list(case["bc"]) + list(case.get("bc_kinds", []))):
        c.bc_type[s], c.bc_density[s], c.bc_pstatic[s] = t, dens, ps
        for a in range(3):
            c.bc_velocity[s][a] = vel[a]
    c.threads = threads
    for flag, vec, key in (("external_force", "sigma", "external_force"),
                           ("uniform_acceleration", "acceleration", "uniform_acceleration")):
        v = case.get(key)
        setattr(c, flag, int(v is not None))
        for a in range(3):
            getattr(c, vec)[a] = v[a] if v is not None else 0.0
    c.viscous = int(bool(case.get("viscous", False)))
    c.viscosity = float(case.get("viscosity", 0.0))
    c._markers = []
    if case.get("bc_split"):
        for side, arr in split_markers(case).items():
            c._markers.append(arr)
            c.bc_marker[side] = arr.ctypes.data_as(C.POINTER(C.c_ubyte))
    return c


def split_markers(case: dict) -> dict:
    """Per-face markers of the case's split sides: case["bc_split"] maps a
    side (0..5) to (axis, pos, kind_lo, kind_hi); a boundary face whose
    centre lies below pos along the tangential `axis` takes kind_lo, the
    others kind_hi.  Face centres' tangential coordinates are the cell
    centres of the oracle's own grid (the reference evaluates its marker
    function at the face centre, ExplicitRungeKuttaFVM.h:1193-1209)."""
    nd = case["ndims"]
    x, _, y, _, z, _ = grid(dict(case, bc_split={}))
    centres = [x[1:-1], y[1:-1] if nd > 1 else y[:1], z[1:-1] if nd > 2 else z[:1]]
    out = {}
    for side, (axis, pos, lo, hi) in case["bc_split"].items():
        a = side // 2
        t = [b for b in range(3) if b != a]
        if axis not in t:
            raise ValueError("the split axis must be tangential to the side")
        cp, cq = centres[t[0]], centres[t[1]]
        coord = cp[:, None] if axis == t[0] else cq[None, :]
        m = np.where(coord < pos, lo, hi) * np.ones((len(cp), len(cq)), dtype=np.int64)
        out[side] = np.ascontiguousarray(m.T.reshape(-1), dtype=np.uint8)
    return out


def dims(case: dict):
    nxa = case["nx"] + 2
    nya = case["ny"] + 2 if case["ndims"] > 1 else 1
    nza = case["nz"] + 2 if case["ndims"] > 2 else 1
    return nxa, nya, nza


def interior_slices(case: dict):
    nd = case["ndims"]
    return (slice(1, -1) if nd > 2 else slice(0, 1), slice(1, -1) if nd > 1 else slice(0, 1), slice(1, -1))


def embed(case: dict, interior: np.ndarray) -> np.ndarray:
    """Interior cells (nz, ny, nx, 5) -> the reference's full values array
    (nza, nya, nxa, 5) with zero ghosts."""
    nxa, nya, nza = dims(case)
    full = np.zeros((nza, nya, nxa, 5))
    full[interior_slices(case)] = interior.reshape(full[interior_slices(case)].shape)
    return full


def grid(case: dict):
    nxa, nya, nza = dims(case)
    arrs = [np.zeros(n) for n in (nxa, nxa, nya, nya, nza, nza)]
    cfg = to_struct(case)
    lib().orc_grid(C.byref(cfg), *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs])
    return arrs


def advance(case: dict, full: np.ndarray, n_steps: int = -1, info: dict | None = None, threads: int = 0):
    """Advance a full values array (with ghosts).  n_steps < 0 runs the
    reference's Run loop (MaxIteration / MaxTime).  Returns (values, info)."""
    vals = np.ascontiguousarray(full, dtype=np.float64).copy()
    cfg = to_struct(case, threads)
    si = OrcStepInfo()
    info = info or {}
    si.iteration = info.get("iteration", 0)
    si.time = info.get("time", 0.0)
    si.next_solution_time = info.get("next_solution_time", case["save_solution_time"])
    si.next_slice_time = info.get("next_slice_time", case["save_slice_time"])
    rc = lib().orc_advance(C.byref(cfg), vals.ctypes.data_as(C.POINTER(C.c_double)), n_steps, C.byref(si))
    if rc != 0:
        raise RuntimeError(f"oracle failed rc={rc}")
    out = dict(iteration=si.iteration, time=si.time, dt=si.dt, next_solution_time=si.next_solution_time,
               next_slice_time=si.next_slice_time, residual=list(si.residual))
    return vals, out


SCENARIO_SHOCK_TUBE, SCENARIO_SHEAR_LAYER, SCENARIO_BLAST, SCENARIO_QUADRANTS = 0, 1, 2, 3


def fill_scenario(case: dict, scenario: int, seed: int, params, threads: int = 0) -> np.ndarray:
    """The seeded initial state of a benchmark scenario, interior cells as
    (nz, ny, nx, 5): the same values the product's ts_fill_scenario writes."""
    nx = case["nx"]
    ny = case["ny"] if case["ndims"] > 1 else 1
    nz = case["nz"] if case["ndims"] > 2 else 1
    out = np.empty((nz, ny, nx, 5))
    p = np.ascontiguousarray(params, dtype=np.float64)
    cfg = to_struct(case, threads)
    rc = lib().orc_fill_scenario(C.byref(cfg), scenario, seed, p.ctypes.data_as(C.POINTER(C.c_double)), len(p),
                                 out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise RuntimeError(f"orc_fill_scenario failed rc={rc}")
    return out


def exact_riemann(gamma, p_inf, left, right, s):
    """Exact (rho, u, p) at x/t = s for primitive left/right states."""
    r, u, p = C.c_double(), C.c_double(), C.c_double()
    lib().orc_exact_riemann(gamma, p_inf, *left, *right, s, C.byref(r), C.byref(u), C.byref(p))
    return r.value, u.value, p.value


# --------------------------------------------------------------------------
# Reference driver (only where the reference sources were built)
# --------------------------------------------------------------------------

def ref_available() -> bool:
    return os.path.exists(REF_RUN)


def _ref_config_text(case: dict, ic_path: str, out_path: str, toro: int = 0, steps: int = -1,
                     extra: list | None = None) -> str:
    lines = [f"ndims {case['ndims']}", f"nx {case['nx']}", f"ny {case['ny']}", f"nz {case['nz']}"]
    for a, n in enumerate("xyz"):
        lines.append(f"periodic_{n} {int(case['periodic'][a])}")
        lines.append(f"l{n} {case['length'][a]!r}")
        blocks = case["blocks"].get(a, [])
        if blocks:
            lines.append(f"blocks_{n} {len(blocks)} " + " ".join(f"{p!r} {q!r} {c}" for p, q, c in blocks))
    lines += [f"gamma {case['gamma']!r}", f"recon {case['recon']}", f"limiter {case['limiter']}",
              f"solver {case['solver']}", f"eps {case['eps']!r}", f"cfl {case['cfl']!r}", "rk_order 1",
              f"max_iter {case['max_iter']}", f"max_time {case['max_time']!r}",
              f"save_solution_time {case['save_solution_time']!r}", f"save_slice_time {case['save_slice_time']!r}"]
    for s, name in enumerate(["bc_xl", "bc_xr", "bc_yl", "bc_yr", "bc_zl", "bc_zr"]):
        t, dens, vel, ps = case["bc"][s]
        lines.append(f"{name} {t} {dens!r} {vel[0]!r} {vel[1]!r} {vel[2]!r} {ps!r}")
    for m, (t, dens, vel, ps) in enumerate(case.get("bc_kinds", [])):
        lines.append(f"bc_kind {m} {t} {dens!r} {vel[0]!r} {vel[1]!r} {vel[2]!r} {ps!r}")
    for side, (axis, pos, lo, hi) in sorted(case.get("bc_split", {}).items()):
        lines.append(f"bc_split {side} {axis} {pos!r} {lo} {hi}")
    if case.get("external_force") is not None:
        lines.append("external_force " + " ".join(repr(float(v)) for v in case["external_force"]))
    if case.get("uniform_acceleration") is not None:
        lines.append("uniform_acceleration " + " ".join(repr(float(v)) for v in case["uniform_acceleration"]))
    if case.get("viscous"):
        lines.append("viscous 1")
    if case.get("viscosity", 0.0):
        lines.append("viscosity " + repr(float(case["viscosity"])))
    lines += [f"ic_file {ic_path}", f"out_file {out_path}"]
    if toro:
        lines.append(f"toro {toro}")
    if steps >= 0:
        lines.append(f"steps {steps}")
    lines += extra or []
    return "\n".join(lines) + "\n"


def read_ref_output(path: str) -> dict:
    with open(path, "rb") as f:
        data = f.read()
    hdr = struct.unpack_from("<8i", data, 0)
    sc = struct.unpack_from("<4d", data, 32)
    off = 64
    arrs = []
    while off < len(data):
        (n,) = struct.unpack_from("<q", data, off)
        off += 8
        arrs.append(np.frombuffer(data, dtype="<f8", count=n, offset=off).copy())
        off += 8 * n
    nd, nxa, nya, nza = hdr[1], hdr[2], hdr[3], hdr[4]
    out = dict(ndims=nd, nxa=nxa, nya=nya, nza=nza, iteration=hdr[5], time=sc[0], dt=sc[1], seconds=sc[2],
               x=arrs[0], hx=arrs[1], y=arrs[2], hy=arrs[3], z=arrs[4], hz=arrs[5], volumes=arrs[6],
               initial=arrs[7].reshape(nza, nya, nxa, 5), values=arrs[8].reshape(nza, nya, nxa, 5),
               residual=arrs[9])
    if hdr[6]:
        out["exact"] = arrs[10].reshape(-1, 5)
        out["errors"] = arrs[11]
    return out


def run_reference(case: dict, interior_ic: np.ndarray | None, toro: int = 0, steps: int = -1,
                  load_solution: bytes | None = None, save_solution: bool = False, save_tecplot: bool = False,
                  molar_mass: float | None = None, gas_constant: float | None = None) -> dict:
    """Run the reference's own ExplicitRungeKuttaFVM on this case (in a scratch
    directory, since the reference writes history.dat to its cwd).  Optionally
    Kernel::LoadSolution a file before stepping, and return the bytes of
    Kernel::SaveSolution / SaveSolutionToTecplot after it."""
    if not ref_available():
        raise RuntimeError("oracle/_ref/ref_run is not built")
    with tempfile.TemporaryDirectory() as d:
        ic = os.path.join(d, "ic.bin")
        out = os.path.join(d, "out.bin")
        if interior_ic is not None:
            np.ascontiguousarray(interior_ic, dtype="<f8").tofile(ic)
        extra = []
        if load_solution is not None:
            with open(os.path.join(d, "load.bin"), "wb") as f:
                f.write(load_solution)
            extra.append(f"load_solution {os.path.join(d, 'load.bin')}")
        if save_solution:
            extra.append(f"save_solution {os.path.join(d, 'sol.bin')}")
        if save_tecplot:
            extra.append(f"save_tecplot {os.path.join(d, 'sol.dat')}")
        if molar_mass is not None:
            extra.append(f"molar_mass {molar_mass!r}")
        if gas_constant is not None:
            extra.append(f"gas_constant {gas_constant!r}")
        cfg = os.path.join(d, "case.txt")
        with open(cfg, "w") as f:
            f.write(_ref_config_text(case, ic, out, toro, steps, extra))
        subprocess.run([REF_RUN, cfg], cwd=d, check=True, stdout=subprocess.DEVNULL)
        r = read_ref_output(out)
        for key, name, flag in (("solution_bytes", "sol.bin", save_solution),
                                ("tecplot_bytes", "sol.dat", save_tecplot)):
            if flag:
                with open(os.path.join(d, name), "rb") as f:
                    r[key] = f.read()
        return r
