"""ctypes binding of the C ABI in include/ts_fvm.h.

The library is the in-tree ``libtsfvm.so`` built by :mod:`turbostructred_gb300.build`.
Loading fails loudly when it is missing: there is no CPU fallback.

Problems are described by the same plain ``dict`` keys the reference's
KernelConfiguration uses (ndims, nx, ny, nz, periodic, length, blocks, gamma,
recon, limiter, solver, eps, cfl, max_iter, max_time, bc ...), see
:func:`make_case`.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtsfvm.so")

ABI_VERSION = 5
MAX_BC_KINDS = 8

# enum values (include/ts_fvm.h)
RECON_PWC, RECON_LINEAR2, RECON_ENO2, RECON_LINEAR2_LIM = 0, 1, 2, 3
RS_GODUNOV, RS_ROE, RS_NONE, RS_HLLC = 0, 1, 2, 3
LIM_BJ, LIM_VENKAT = 0, 1
BC_WALL, BC_SYMMETRY, BC_MOVING_WALL, BC_SUBSONIC_INLET, BC_SUBSONIC_OUTLET, BC_NATURAL = range(6)
EOS_IDEAL, EOS_STIFFENED = 0, 1
PRECISION_FP64, PRECISION_MIXED = 0, 1
LAYOUT_INTERIOR, LAYOUT_WITH_GHOSTS = 0, 1
SCENARIO_SHOCK_TUBE, SCENARIO_SHEAR_LAYER, SCENARIO_BLAST, SCENARIO_QUADRANTS = 0, 1, 2, 3
HEALTH_NAN, HEALTH_NEG_DENSITY, HEALTH_NEG_PRESSURE, HEALTH_RIEMANN = 1, 2, 4, 8

STATUS = {0: "ok", 1: "invalid", 2: "unsupported", 3: "cuda", 4: "no_memory", 5: "numeric",
          6: "timeout", 7: "busy", 8: "not_found"}


class TsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class BlockNode(C.Structure):
    _fields_ = [("pos", C.c_double), ("q_com", C.c_double), ("n_cells", C.c_int32), ("reserved", C.c_int32)]


class BcConfig(C.Structure):
    _fields_ = [("type", C.c_int32), ("reserved", C.c_int32), ("density", C.c_double),
                ("velocity", C.c_double * 3), ("pstatic", C.c_double), ("temperature", C.c_double)]


class Config(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("n_dims", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32),
        ("nz", C.c_int32), ("periodic", C.c_int32 * 3), ("length", C.c_double * 3),
        ("n_blocks", C.c_int32 * 3), ("reserved0", C.c_int32), ("blocks", C.POINTER(BlockNode) * 3),
        ("gamma", C.c_double), ("eos", C.c_int32), ("reserved1", C.c_int32), ("p_inf", C.c_double),
        ("reconstruction", C.c_int32), ("riemann_solver", C.c_int32), ("limiter", C.c_int32),
        ("rk_order", C.c_int32), ("cfl", C.c_double), ("eps", C.c_double),
        ("max_iteration", C.c_int32), ("reserved2", C.c_int32), ("max_time", C.c_double),
        ("save_solution_time", C.c_double), ("save_slice_time", C.c_double),
        ("bc", BcConfig * 6), ("precision", C.c_int32), ("device", C.c_int32),
        ("external_force", C.c_int32), ("uniform_acceleration", C.c_int32),
        ("sigma", C.c_double * 3), ("acceleration", C.c_double * 3),
        ("viscous", C.c_int32), ("residual_norms", C.c_int32), ("viscosity", C.c_double),
        ("n_bc_kinds", C.c_int32), ("reserved4", C.c_int32), ("bc_kinds", BcConfig * MAX_BC_KINDS),
        ("bc_marker", C.POINTER(C.c_uint8) * 6),
    ]


class StepInfo(C.Structure):
    _fields_ = [("iteration", C.c_int32), ("health", C.c_uint32), ("time", C.c_double), ("dt", C.c_double),
                ("next_solution_time", C.c_double), ("next_slice_time", C.c_double),
                ("residual", C.c_double * 5)]

    def as_dict(self):
        return dict(iteration=self.iteration, health=self.health, time=self.time, dt=self.dt,
                    next_solution_time=self.next_solution_time, next_slice_time=self.next_slice_time,
                    residual=list(self.residual))


MAX_KERNELS = 16


class Timing(C.Structure):
    _fields_ = [("total_ms", C.c_double), ("n_kernels", C.c_int32), ("launches", C.c_int32),
                ("kernel_ms", C.c_double * MAX_KERNELS), ("kernel_name", (C.c_char * 32) * MAX_KERNELS)]

    def as_dict(self):
        return dict(total_ms=self.total_ms, launches=self.launches,
                    kernels={self.kernel_name[k].value.decode(): self.kernel_ms[k] for k in range(self.n_kernels)})


SERVE_FIFO, SERVE_SHORTEST_FIRST = 0, 1


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("order", C.c_int32), ("memory_budget", C.c_size_t),
                ("max_cells", C.c_int64), ("max_active", C.c_int32), ("reserved", C.c_int32),
                ("chunk_ms", C.c_double)]


class RequestTimes(C.Structure):
    _fields_ = [("submit_s", C.c_double), ("admit_s", C.c_double), ("finish_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "admitted", "completed", "rejected", "queued", "active",
                                         "stages", "launches")] + \
               [(n, C.c_double) for n in ("cell_updates", "busy_s", "admit_s", "retire_s", "latency_p50_ms",
                                          "latency_p99_ms",
                                          "latency_max_ms", "wait_p50_ms", "wait_p99_ms")] + \
               [("bytes_budget", C.c_size_t), ("bytes_in_use", C.c_size_t), ("worker_status", C.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


EXPORTS = [
    "ts_create", "ts_destroy", "ts_set_state", "ts_set_state_device", "ts_get_state", "ts_get_state_device",
    "ts_step", "ts_step_timed", "ts_run", "ts_set_tile",
    "ts_get_step_info", "ts_set_step_info", "ts_synchronize", "ts_grid_coordinates", "ts_state_doubles",
    "ts_fill_scenario", "ts_hash_uniform", "ts_last_error", "ts_status_string",
    "ts_batch_create", "ts_batch_destroy", "ts_batch_add", "ts_batch_problem_bytes", "ts_batch_step",
    "ts_batch_run", "ts_batch_finished", "ts_batch_get", "ts_batch_remove", "ts_batch_set_tile",
    "ts_batch_autotune", "ts_batch_stats", "ts_batch_launch", "ts_batch_wait", "ts_batch_set_tail",
    "ts_server_create", "ts_server_destroy", "ts_server_submit", "ts_server_wait", "ts_server_drain",
    "ts_server_stats_get",
    "ts_save_solution", "ts_load_solution", "ts_save_tecplot", "ts_wait_writes", "ts_write_solution_file",
    "ts_read_solution_file", "ts_write_tecplot_file",
]

_lib = None


def load(path: str = LIB_PATH):
    """Load the in-tree CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run turbostructred_gb300.build.build() first")
    L = C.CDLL(path)
    P = C.POINTER
    L.ts_create.argtypes = [P(Config), P(C.c_void_p)]
    L.ts_destroy.argtypes = [C.c_void_p]
    L.ts_destroy.restype = None
    L.ts_set_state.argtypes = [C.c_void_p, P(C.c_double), C.c_int32]
    L.ts_set_state_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
    L.ts_get_state_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
    L.ts_get_state.argtypes = [C.c_void_p, P(C.c_double), C.c_int32]
    L.ts_step.argtypes = [C.c_void_p, C.c_int32, P(StepInfo)]
    L.ts_step_timed.argtypes = [C.c_void_p, C.c_int32, P(StepInfo), P(Timing)]
    L.ts_run.argtypes = [C.c_void_p, P(StepInfo)]
    L.ts_get_step_info.argtypes = [C.c_void_p, P(StepInfo)]
    L.ts_set_step_info.argtypes = [C.c_void_p, P(StepInfo)]
    L.ts_synchronize.argtypes = [C.c_void_p]
    L.ts_set_tile.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
    L.ts_set_tile.restype = C.c_int
    L.ts_grid_coordinates.argtypes = [P(Config)] + [P(C.c_double)] * 6
    L.ts_state_doubles.argtypes = [P(Config), C.c_int32]
    L.ts_state_doubles.restype = C.c_size_t
    L.ts_fill_scenario.argtypes = [P(Config), C.c_int32, C.c_uint64, P(C.c_double), C.c_int32, P(C.c_double)]
    L.ts_hash_uniform.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int64]
    L.ts_hash_uniform.restype = C.c_double
    L.ts_batch_create.argtypes = [C.c_int32, C.c_size_t, P(C.c_void_p)]
    L.ts_batch_destroy.argtypes = [C.c_void_p]
    L.ts_batch_destroy.restype = None
    L.ts_batch_add.argtypes = [C.c_void_p, P(Config), P(C.c_double), P(C.c_int32)]
    L.ts_batch_problem_bytes.argtypes = [P(Config)]
    L.ts_batch_problem_bytes.restype = C.c_size_t
    L.ts_batch_step.argtypes = [C.c_void_p, C.c_int32]
    L.ts_batch_run.argtypes = [C.c_void_p, C.c_int32, P(C.c_int32)]
    L.ts_batch_finished.argtypes = [C.c_void_p, P(C.c_int32), C.c_int32, P(C.c_int32)]
    L.ts_batch_get.argtypes = [C.c_void_p, C.c_int32, P(C.c_double), P(StepInfo)]
    L.ts_batch_remove.argtypes = [C.c_void_p, C.c_int32]
    L.ts_batch_set_tile.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.ts_batch_set_tail.argtypes = [C.c_void_p, C.c_int32]
    L.ts_batch_autotune.argtypes = [C.c_void_p, C.c_int32, P(C.c_int32), P(C.c_int32), P(C.c_int32)]
    L.ts_batch_stats.argtypes = [C.c_void_p, P(C.c_double), P(C.c_int64), P(C.c_int64)]
    L.ts_batch_launch.argtypes = [C.c_void_p, C.c_int32]
    L.ts_batch_wait.argtypes = [C.c_void_p, P(C.c_int32)]
    L.ts_batch_launch.restype = C.c_int
    L.ts_batch_wait.restype = C.c_int
    for name in ("ts_batch_create", "ts_batch_add", "ts_batch_step", "ts_batch_run", "ts_batch_finished",
                 "ts_batch_get", "ts_batch_remove", "ts_batch_set_tile", "ts_batch_autotune", "ts_batch_stats"):
        getattr(L, name).restype = C.c_int
    L.ts_server_create.argtypes = [P(ServerConfig), P(C.c_void_p)]
    L.ts_server_destroy.argtypes = [C.c_void_p]
    L.ts_server_destroy.restype = None
    L.ts_server_submit.argtypes = [C.c_void_p, P(Config), P(C.c_double), C.c_int32, P(C.c_int32)]
    L.ts_server_wait.argtypes = [C.c_void_p, C.c_int32, C.c_int32, P(C.c_double), P(StepInfo), P(RequestTimes)]
    L.ts_server_drain.argtypes = [C.c_void_p, C.c_int32]
    L.ts_server_stats_get.argtypes = [C.c_void_p, P(ServerStats)]
    for name in ("ts_server_create", "ts_server_submit", "ts_server_wait", "ts_server_drain", "ts_server_stats_get"):
        getattr(L, name).restype = C.c_int
    L.ts_save_solution.argtypes = [C.c_void_p, C.c_char_p]
    L.ts_load_solution.argtypes = [C.c_void_p, C.c_char_p]
    L.ts_save_tecplot.argtypes = [C.c_void_p, C.c_char_p, C.c_double, C.c_double, C.c_int32]
    L.ts_wait_writes.argtypes = [C.c_void_p]
    L.ts_write_solution_file.argtypes = [P(Config), P(C.c_double), C.c_double, C.c_char_p]
    L.ts_read_solution_file.argtypes = [P(Config), C.c_char_p, P(C.c_double), P(C.c_double)]
    L.ts_write_tecplot_file.argtypes = [P(Config), P(C.c_double), C.c_double, C.c_double, C.c_double, C.c_char_p]
    for name in ("ts_save_solution", "ts_load_solution", "ts_save_tecplot", "ts_wait_writes",
                 "ts_write_solution_file", "ts_read_solution_file", "ts_write_tecplot_file"):
        getattr(L, name).restype = C.c_int
    L.ts_last_error.restype = C.c_char_p
    L.ts_status_string.restype = C.c_char_p
    for name in ("ts_create", "ts_set_state", "ts_set_state_device", "ts_get_state", "ts_get_state_device",
                 "ts_step", "ts_step_timed", "ts_run",
                 "ts_get_step_info", "ts_set_step_info", "ts_synchronize", "ts_grid_coordinates",
                 "ts_fill_scenario"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(status: int):
    if status != 0:
        raise TsError(status, load().ts_last_error().decode())


def make_case(**kw) -> dict:
    """Problem description; defaults follow KernelConfiguration.h:21-93."""
    case = dict(ndims=1, nx=1, ny=1, nz=1, periodic=(1, 1, 1), length=(1.0, 1.0, 1.0), blocks={},
                gamma=1.4, eos=EOS_IDEAL, p_inf=0.0, recon=RECON_PWC, limiter=LIM_BJ, solver=RS_ROE,
                eps=0.0, cfl=0.25, max_iter=1000, max_time=1.0, save_solution_time=0.0,
                save_slice_time=0.0, bc=[(BC_NATURAL, 0.0, (0.0, 0.0, 0.0), 0.0)] * 6,
                external_force=None, uniform_acceleration=None, viscous=False, viscosity=0.0,
                residual_norms=False, bc_kinds=[], bc_split={})
    case.update(kw)
    return case


def to_config(case: dict, precision: int = PRECISION_FP64, device: int = 0):
    """Returns (Config, keepalive) -- keepalive holds the block arrays."""
    c = Config()
    c.abi_version = ABI_VERSION
    c.n_dims, c.nx, c.ny, c.nz = case["ndims"], case["nx"], case["ny"], case["nz"]
    keep = []
    for a in range(3):
        c.periodic[a] = int(case["periodic"][a])
        c.length[a] = case["length"][a]
        blocks = case.get("blocks", {}).get(a, [])
        if blocks:
            arr = (BlockNode * len(blocks))()
            for b, (pos, q, n) in enumerate(blocks):
                arr[b].pos, arr[b].q_com, arr[b].n_cells = pos, q, n
            keep.append(arr)
            c.n_blocks[a] = len(blocks)
            c.blocks[a] = C.cast(arr, C.POINTER(BlockNode))
    c.gamma, c.eos, c.p_inf = case["gamma"], case.get("eos", EOS_IDEAL), case.get("p_inf", 0.0)
    c.reconstruction, c.riemann_solver, c.limiter = case["recon"], case["solver"], case["limiter"]
    c.rk_order = 1
    c.cfl, c.eps = case["cfl"], case["eps"]
    c.max_iteration, c.max_time = case["max_iter"], case["max_time"]
    c.save_solution_time = case.get("save_solution_time", 0.0)
    c.save_slice_time = case.get("save_slice_time", 0.0)
    for s, (t, dens, vel, ps) in enumerate(case["bc"]):
        c.bc[s].type, c.bc[s].density, c.bc[s].pstatic = t, dens, ps
        for a in range(3):
            c.bc[s].velocity[a] = vel[a]
    c.precision, c.device = precision, device
    # source terms: None (off) or a 3-vector
    for flag, vec, key in (("external_force", "sigma", "external_force"),
                           ("uniform_acceleration", "acceleration", "uniform_acceleration")):
        v = case.get(key)
        setattr(c, flag, int(v is not None))
        for a in range(3):
            getattr(c, vec)[a] = v[a] if v is not None else 0.0
    c.viscous = int(bool(case.get("viscous", False)))
    c.viscosity = float(case.get("viscosity", 0.0))
    c.residual_norms = int(bool(case.get("residual_norms", False)))
    # position-dependent sides: extra BC kinds and per-face markers
    kinds = case.get("bc_kinds", [])
    c.n_bc_kinds = len(kinds)
    for m, (t, dens, vel, ps) in enumerate(kinds):
        c.bc_kinds[m].type, c.bc_kinds[m].density, c.bc_kinds[m].pstatic = t, dens, ps
        for a in range(3):
            c.bc_kinds[m].velocity[a] = vel[a]
    if case.get("bc_split"):
        for side, arr in split_markers(case, c).items():
            keep.append(arr)
            c.bc_marker[side] = arr.ctypes.data_as(C.POINTER(C.c_uint8))
    return c, keep


def split_markers(case: dict, cfg=None) -> dict:
    """Per-face marker arrays of the case's split sides.  case["bc_split"]
    maps a side (0..5: x-, x+, y-, y+, z-, z+) to (axis, pos, kind_lo,
    kind_hi): a boundary face whose centre's coordinate along the tangential
    `axis` is below pos takes bc_kinds[kind_lo], the others
    bc_kinds[kind_hi] -- a marker function like the reference's
    DomainBCinfo::getMarker, evaluated at the faces' centres.  Faces are
    numbered as ts_config.bc_marker expects (x sides j + ny k, y sides
    i + nx k, z sides i + nx j)."""
    if cfg is None:
        cfg, _ = to_config(dict(case, bc_split={}))
    nd = case["ndims"]
    nx, ny, nz = case["nx"], case["ny"] if nd > 1 else 1, case["nz"] if nd > 2 else 1
    arrs = [np.zeros(n) for n in (nx + 2, nx + 2, (ny + 2) if nd > 1 else 1, (ny + 2) if nd > 1 else 1,
                                  (nz + 2) if nd > 2 else 1, (nz + 2) if nd > 2 else 1)]
    P = C.POINTER(C.c_double)
    check(load().ts_grid_coordinates(C.byref(cfg), *[a.ctypes.data_as(P) for a in arrs]))
    centres = [arrs[0][1:-1] if nd >= 1 else arrs[0], arrs[2][1:-1] if nd > 1 else arrs[2][:1],
               arrs[4][1:-1] if nd > 2 else arrs[4][:1]]
    out = {}
    for side, (axis, pos, lo, hi) in case["bc_split"].items():
        a = side // 2
        t = [b for b in range(3) if b != a]          # tangential axes, lower first
        if axis not in t:
            raise ValueError("the split axis must be tangential to the side")
        # face (p, q): p along t[0] (fastest), q along t[1]
        cp, cq = centres[t[0]], centres[t[1]]
        coord = cp[:, None] if axis == t[0] else cq[None, :]
        m = np.where(coord < pos, lo, hi) * np.ones((len(cp), len(cq)), dtype=np.int64)
        out[side] = np.ascontiguousarray(m.T.reshape(-1), dtype=np.uint8)
    return out


def interior_shape(case: dict):
    nd = case["ndims"]
    return (case["nz"] if nd > 2 else 1, case["ny"] if nd > 1 else 1, case["nx"], 5)


def ghost_shape(case: dict):
    nd = case["ndims"]
    return (case["nz"] + 2 if nd > 2 else 1, case["ny"] + 2 if nd > 1 else 1, case["nx"] + 2, 5)


def grid_coordinates(case: dict):
    cfg, keep = to_config(case)
    nx = case["nx"] + 2
    ny = case["ny"] + 2 if case["ndims"] > 1 else 1
    nz = case["nz"] + 2 if case["ndims"] > 2 else 1
    arrs = [np.zeros(n) for n in (nx, nx, ny, ny, nz, nz)]
    check(load().ts_grid_coordinates(C.byref(cfg), *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]))
    return arrs


def fill_scenario(case: dict, scenario: int, seed: int, params) -> np.ndarray:
    """Synthetic initial state (interior cells, shape (nz, ny, nx, 5))."""
    cfg, keep = to_config(case)
    out = np.zeros(interior_shape(case))
    p = (C.c_double * len(params))(*params)
    check(load().ts_fill_scenario(C.byref(cfg), scenario, seed, p, len(params),
                                  out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


GAS_CONSTANT = 8.3144598  # KernelConfiguration::UniversalGasConstant default


def write_solution_file(case: dict, values: np.ndarray, time: float, path: str):
    """Kernel::SaveSolution's binary layout from a host state (interior cells)."""
    cfg, keep = to_config(case)
    v = np.ascontiguousarray(values, dtype=np.float64)
    check(load().ts_write_solution_file(C.byref(cfg), v.ctypes.data_as(C.POINTER(C.c_double)), time,
                                        os.fsencode(path)))


def read_solution_file(case: dict, path: str):
    cfg, keep = to_config(case)
    out = np.empty(interior_shape(case))
    t = C.c_double()
    check(load().ts_read_solution_file(C.byref(cfg), os.fsencode(path), out.ctypes.data_as(C.POINTER(C.c_double)),
                                       C.byref(t)))
    return out, t.value


def write_tecplot_file(case: dict, values: np.ndarray, time: float, path: str, molar_mass: float = 0.0,
                       gas_constant: float = GAS_CONSTANT):
    cfg, keep = to_config(case)
    v = np.ascontiguousarray(values, dtype=np.float64)
    check(load().ts_write_tecplot_file(C.byref(cfg), v.ctypes.data_as(C.POINTER(C.c_double)), time, molar_mass,
                                       gas_constant, os.fsencode(path)))


class Solver:
    """One device-resident domain driven through the C ABI."""

    def __init__(self, case: dict, precision: int = PRECISION_FP64, device: int = 0):
        self.case = case
        self.lib = load()
        cfg, self._keep = to_config(case, precision, device)
        self._cfg = cfg
        h = C.c_void_p()
        check(self.lib.ts_create(C.byref(cfg), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.ts_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, values: np.ndarray, layout: int = LAYOUT_INTERIOR):
        v = np.ascontiguousarray(values, dtype=np.float64)
        check(self.lib.ts_set_state(self.h, v.ctypes.data_as(C.POINTER(C.c_double)), layout))

    def set_state_device(self, ptr: int, layout: int = LAYOUT_INTERIOR):
        """The state from device memory at `ptr`; whatever wrote it must have
        completed (e.g. torch.cuda.synchronize()): the solver reads it on its
        own stream."""
        check(self.lib.ts_set_state_device(self.h, C.c_void_p(ptr), layout))

    def get_state(self, layout: int = LAYOUT_INTERIOR, out: np.ndarray | None = None) -> np.ndarray:
        shape = interior_shape(self.case) if layout == LAYOUT_INTERIOR else ghost_shape(self.case)
        if out is None:
            out = np.empty(shape)
        check(self.lib.ts_get_state(self.h, out.ctypes.data_as(C.POINTER(C.c_double)), layout))
        return out

    def get_state_device(self, ptr: int, layout: int = LAYOUT_INTERIOR):
        """The state into device memory at `ptr` (on the solver's device), in
        the layout of get_state."""
        check(self.lib.ts_get_state_device(self.h, C.c_void_p(ptr), layout))

    def step(self, n: int = 1) -> dict:
        si = StepInfo()
        check(self.lib.ts_step(self.h, n, C.byref(si)))
        return si.as_dict()

    def step_timed(self, n: int):
        """n steps with CUDA events on the library's stream: (info, timing)."""
        si, tm = StepInfo(), Timing()
        check(self.lib.ts_step_timed(self.h, n, C.byref(si), C.byref(tm)))
        return si.as_dict(), tm.as_dict()

    def run(self) -> dict:
        si = StepInfo()
        check(self.lib.ts_run(self.h, C.byref(si)))
        return si.as_dict()

    def info(self) -> dict:
        si = StepInfo()
        check(self.lib.ts_get_step_info(self.h, C.byref(si)))
        return si.as_dict()

    def set_info(self, **kw):
        si = StepInfo()
        check(self.lib.ts_get_step_info(self.h, C.byref(si)))
        for k, v in kw.items():
            setattr(si, k, v)
        check(self.lib.ts_set_step_info(self.h, C.byref(si)))

    def synchronize(self):
        check(self.lib.ts_synchronize(self.h))

    def set_tile(self, tx: int, ty: int, z_chunks: int = 0):
        check(self.lib.ts_set_tile(self.h, tx, ty, z_chunks))

    def save_solution(self, path: str):
        check(self.lib.ts_save_solution(self.h, os.fsencode(path)))

    def load_solution(self, path: str):
        check(self.lib.ts_load_solution(self.h, os.fsencode(path)))

    def save_tecplot(self, path: str, molar_mass: float = 0.0, gas_constant: float = GAS_CONSTANT,
                     asynchronous: bool = False):
        check(self.lib.ts_save_tecplot(self.h, os.fsencode(path), molar_mass, gas_constant, int(asynchronous)))

    def wait_writes(self):
        check(self.lib.ts_wait_writes(self.h))


def batch_problem_bytes(case: dict) -> int:
    cfg, keep = to_config(case, PRECISION_MIXED)
    return int(load().ts_batch_problem_bytes(C.byref(cfg)))


class Batch:
    """Independent 1D/2D problems advanced together (mixed precision), each
    under Kernel::Run termination rules with its own dt."""

    def __init__(self, memory_budget: int, device: int = 0):
        self.lib = load()
        b = C.c_void_p()
        check(self.lib.ts_batch_create(device, memory_budget, C.byref(b)))
        self.b = b
        self.cases = {}

    def close(self):
        if self.b:
            self.lib.ts_batch_destroy(self.b)
            self.b = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, case: dict, values: np.ndarray) -> int:
        cfg, keep = to_config(case, PRECISION_MIXED)
        v = np.ascontiguousarray(values, dtype=np.float64)
        assert v.size == int(np.prod(interior_shape(case)))
        pid = C.c_int32()
        check(self.lib.ts_batch_add(self.b, C.byref(cfg), v.ctypes.data_as(C.POINTER(C.c_double)), C.byref(pid)))
        self.cases[pid.value] = case
        return pid.value

    def step(self, n: int = 1):
        check(self.lib.ts_batch_step(self.b, n))

    def run(self, max_stages: int = 0) -> int:
        a = C.c_int32()
        check(self.lib.ts_batch_run(self.b, max_stages, C.byref(a)))
        return a.value

    def launch(self, n: int):
        check(self.lib.ts_batch_launch(self.b, n))

    def wait(self) -> int:
        a = C.c_int32()
        check(self.lib.ts_batch_wait(self.b, C.byref(a)))
        return a.value

    def finished(self, cap: int = 1 << 16) -> list:
        ids = (C.c_int32 * cap)()
        n = C.c_int32()
        check(self.lib.ts_batch_finished(self.b, ids, cap, C.byref(n)))
        return list(ids[:n.value])

    def get(self, pid: int, want_state: bool = True):
        si = StepInfo()
        case = self.cases.get(pid)
        out = np.empty(interior_shape(case)) if want_state and case is not None else None
        ptr = out.ctypes.data_as(C.POINTER(C.c_double)) if out is not None else None
        check(self.lib.ts_batch_get(self.b, pid, ptr, C.byref(si)))
        return out, si.as_dict()

    def remove(self, pid: int):
        check(self.lib.ts_batch_remove(self.b, pid))
        self.cases.pop(pid, None)

    def set_tile(self, nd: int, tx: int, ty: int = 1, ctas_per_sm: int = 0):
        check(self.lib.ts_batch_set_tile(self.b, nd, tx, ty, ctas_per_sm))

    def set_tail(self, enable: bool):
        check(self.lib.ts_batch_set_tail(self.b, int(bool(enable))))

    def autotune(self, stages: int = 8):
        tx, ty, ct = C.c_int32(), C.c_int32(), C.c_int32()
        check(self.lib.ts_batch_autotune(self.b, stages, C.byref(tx), C.byref(ty), C.byref(ct)))
        return tx.value, ty.value, ct.value

    def stats(self) -> dict:
        cu, st, la = C.c_double(), C.c_int64(), C.c_int64()
        check(self.lib.ts_batch_stats(self.b, C.byref(cu), C.byref(st), C.byref(la)))
        return dict(cell_updates=cu.value, stages=st.value, launches=la.value)


class Server:
    """Served solves: submit from any thread, a native worker admits them into
    one batch as memory frees up and retires them as they finish."""

    def __init__(self, memory_budget: int, max_active: int = 0, chunk_ms: float = 2.0, device: int = 0,
                 order: int = SERVE_FIFO, max_cells: int = 0):
        self.lib = load()
        cfg = ServerConfig(device=device, order=order, memory_budget=memory_budget, max_cells=max_cells,
                           max_active=max_active, reserved=0, chunk_ms=chunk_ms)
        h = C.c_void_p()
        check(self.lib.ts_server_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.cases = {}

    def close(self):
        if self.h:
            self.lib.ts_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, case: dict, values: np.ndarray, keep_state: bool = True) -> int:
        cfg, keep = to_config(case, PRECISION_MIXED)
        v = np.ascontiguousarray(values, dtype=np.float64)
        assert v.size == int(np.prod(interior_shape(case)))
        rid = C.c_int32()
        check(self.lib.ts_server_submit(self.h, C.byref(cfg), v.ctypes.data_as(C.POINTER(C.c_double)),
                                        int(keep_state), C.byref(rid)))
        self.cases[rid.value] = (case, keep_state)
        return rid.value

    def wait(self, rid: int, timeout_ms: int = -1):
        """(state or None, step info, times) of a finished request."""
        case, kept = self.cases.get(rid, (None, False))
        out = np.empty(interior_shape(case)) if kept else None
        si, tm = StepInfo(), RequestTimes()
        ptr = out.ctypes.data_as(C.POINTER(C.c_double)) if out is not None else None
        check(self.lib.ts_server_wait(self.h, rid, timeout_ms, ptr, C.byref(si), C.byref(tm)))
        self.cases.pop(rid, None)
        return out, si.as_dict(), dict(submit_s=tm.submit_s, admit_s=tm.admit_s, finish_s=tm.finish_s)

    def drain(self, timeout_ms: int = -1):
        check(self.lib.ts_server_drain(self.h, timeout_ms))

    def stats(self) -> dict:
        st = ServerStats()
        check(self.lib.ts_server_stats_get(self.h, C.byref(st)))
        return st.as_dict()
