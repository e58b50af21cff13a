"""Batches of independent 1D/2D problems (include/ts_fvm.h, ts_batch_*).

Each problem in a batch follows Kernel::Run rules with its own dt; the
batch must give every problem the result it would get on its own:
  * bit for bit the same as the problem alone in a batch (same kernel, same
    items: the other problems never touch its arithmetic), whatever else is
    in the batch and whenever it was admitted;
  * equal to FP32 rounding (max relative difference <= 1e-5) to the
    single-problem mixed path, which is a different compiled kernel;
  * within the mixed-precision bar of the FP64 oracle: density L1 <= 1e-5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RHO_L1 = 1e-5
NAT = (5, 0.0, (0.0, 0.0, 0.0), 0.0)
SYM = (1, 0.0, (0.0, 0.0, 0.0), 0.0)
WALL = (0, 0.0, (0.0, 0.0, 0.0), 0.0)
INLET = (3, 1.2, (0.4, 0.0, 0.0), 1.1)
BUDGET = 256 << 20


def l1(a, b, v):
    return float(np.abs(a[..., v] - b[..., v]).sum() / np.abs(b[..., v]).sum())


def relmax(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def mixed_problems(max_time=None, max_iter=None):
    """A mixed set: 1D/2D, PWC/limited/ENO2 reconstruction, Roe/HLLC, ideal
    and stiffened gas, periodic and walled, sizes off the tile multiples."""
    from turbostructred_gb300 import capi
    tube = [0.5, 1.0, 0.0, 1.0, 0.125, 0.0, 0.1]
    stiff = [0.5, 1.5, 0.2, 4.0, 0.8, -0.3, 0.5]
    shear = [2.0, 1.0, 0.5, 2.5, 0.01]
    quad = [1.5, 0.0, 0.0, 1.5, 0.53, 1.2, 0.0, 0.3, 0.14, 1.2, 1.2, 0.03, 0.53, 0.0, 1.2, 0.3]
    specs = [
        (dict(ndims=1, nx=100, periodic=(0, 1, 1), recon=0, solver=1, cfl=0.5, bc=[NAT] * 6), 0, tube, 0.15),
        (dict(ndims=1, nx=257, periodic=(0, 1, 1), recon=3, solver=3, cfl=0.5, bc=[NAT] * 6), 0, tube, 0.1),
        (dict(ndims=1, nx=513, periodic=(0, 1, 1), recon=3, limiter=1, solver=1, cfl=0.5, bc=[NAT] * 6), 0, tube,
         0.05),
        (dict(ndims=1, nx=300, periodic=(0, 1, 1), recon=3, solver=1, gamma=4.4, eos=1, p_inf=6.0, cfl=0.5,
              bc=[NAT] * 6), 0, stiff, 0.02),
        (dict(ndims=1, nx=1000, periodic=(0, 1, 1), recon=2, solver=3, cfl=0.4, bc=[SYM] * 6), 0, tube, 0.03),
        (dict(ndims=2, nx=40, ny=33, periodic=(1, 1, 1), recon=3, solver=3, cfl=0.4), 1, shear, 0.05),
        (dict(ndims=2, nx=64, ny=64, periodic=(1, 1, 1), recon=3, limiter=1, solver=1, cfl=0.4), 1, shear, 0.04),
        (dict(ndims=2, nx=50, ny=37, periodic=(0, 0, 1), recon=3, solver=1, cfl=0.4, bc=[NAT] * 6), 3, quad, 0.05),
        (dict(ndims=2, nx=70, ny=45, periodic=(1, 0, 1), recon=0, solver=3, cfl=0.4,
              bc=[NAT, NAT, SYM, NAT, NAT, NAT]), 1, shear, 0.05),
    ]
    out = []
    for n, (kw, scen, params, t_end) in enumerate(specs):
        kw = dict(kw, max_time=t_end if max_time is None else max_time, max_iter=max_iter or 100000)
        case = capi.make_case(**kw)
        out.append((case, capi.fill_scenario(case, scen, 11 + n, params)))
    return out


def run_batch(problems, budget=BUDGET, tile=None):
    from turbostructred_gb300 import capi
    with capi.Batch(budget) as b:
        if tile:
            b.set_tile(*tile)
        ids = [b.add(c, v) for c, v in problems]
        assert b.run() == 0
        done = b.finished()
        assert sorted(done) == sorted(ids)
        return [b.get(i) for i in ids]


def test_batch_matches_single_problem_path(tslib):
    from turbostructred_gb300 import capi
    probs = mixed_problems(max_time=1e30, max_iter=23)
    res = run_batch(probs)
    for (case, ic), (got, info) in zip(probs, res):
        with capi.Solver(case, precision=capi.PRECISION_MIXED) as s:
            s.set_state(ic)
            sinfo = s.run()
            ref = s.get_state()
        assert info["iteration"] == sinfo["iteration"] == 23
        assert abs(info["time"] - sinfo["time"]) <= 1e-5 * sinfo["time"]
        assert relmax(got, ref) <= 1e-5, (case["ndims"], case["nx"])
        assert info["health"] == 0


def test_batch_close_to_fp64_oracle(tslib, oracle_mod):
    from oracle import oracle as O
    probs = mixed_problems(max_time=1e30, max_iter=17)
    res = run_batch(probs)
    for (case, ic), (got, info) in zip(probs, res):
        ref_full, rinfo = oracle_mod.advance(case, O.embed(case, ic), 17)
        nd = case["ndims"]
        ref = ref_full[(slice(0, 1), slice(1, -1) if nd > 1 else slice(0, 1), slice(1, -1))].reshape(got.shape)
        assert abs(info["time"] - rinfo["time"]) <= 1e-5 * rinfo["time"]
        assert l1(got, ref, 0) <= RHO_L1, (nd, case["nx"], l1(got, ref, 0))


def test_batch_alone_equals_in_mix_bitwise(tslib):
    """A problem's result does not depend on what else is in the batch."""
    probs = mixed_problems()
    mix = run_batch(probs)
    for k in (1, 5, 7):
        alone = run_batch([probs[k]])[0]
        assert alone[1]["iteration"] == mix[k][1]["iteration"]
        assert alone[1]["time"] == mix[k][1]["time"]
        assert np.array_equal(alone[0], mix[k][0])


def test_batch_continuous_admission(tslib):
    """Problems admitted while others run, and finished ones collected and
    removed between stage chunks, still match their runs alone bit for bit."""
    from turbostructred_gb300 import capi
    probs = mixed_problems()
    alone = [run_batch([p])[0] for p in probs]
    results = {}
    with capi.Batch(BUDGET) as b:
        pending = list(range(len(probs)))
        owner = {}
        for _ in range(3):
            k = pending.pop(0)
            owner[b.add(*probs[k])] = k
        while owner:
            b.run(max_stages=7)
            for pid in b.finished():
                results[owner.pop(pid)] = b.get(pid)
                b.remove(pid)
            if pending:
                k = pending.pop(0)
                owner[b.add(*probs[k])] = k
        st = b.stats()
    assert sorted(results) == list(range(len(probs)))
    for k in range(len(probs)):
        assert results[k][1]["iteration"] == alone[k][1]["iteration"]
        assert np.array_equal(results[k][0], alone[k][0]), k
    want = sum(c["nx"] * (c["ny"] if c["ndims"] > 1 else 1) * a[1]["iteration"] for (c, _), a in zip(probs, alone))
    assert st["cell_updates"] == want


def test_batch_midway_reads_and_steps(tslib):
    """ts_batch_step advances every unfinished problem by whole stages, and
    reading a state midway keeps the trajectory to FP32 accuracy."""
    from turbostructred_gb300 import capi
    probs = mixed_problems(max_time=1e30, max_iter=12)
    ref = run_batch(probs)
    with capi.Batch(BUDGET) as b:
        ids = [b.add(c, v) for c, v in probs]
        for _ in range(4):
            b.step(3)
            infos = [b.get(i)[1] for i in ids]
        assert all(inf["iteration"] == 12 for inf in infos)
        b.step(2)  # every problem has finished: no-op
        got = [b.get(i) for i in ids]
    for (g, gi), (r, ri) in zip(got, ref):
        assert gi["iteration"] == 12
        assert relmax(g, r) <= 1e-6


def test_batch_budget_admission(tslib):
    from turbostructred_gb300 import capi
    case = capi.make_case(ndims=2, nx=64, ny=48, periodic=(1, 1, 1), recon=3, cfl=0.4, max_time=0.01)
    ic = capi.fill_scenario(case, 1, 2, [2.0, 1.0, 0.5, 2.5, 0.01])
    per = capi.batch_problem_bytes(case)
    assert per > 64 * 48 * 5 * (2 * 8 + 2 * 4)
    with capi.Batch(3 * per + 4096) as b:
        ids = [b.add(case, ic) for _ in range(3)]
        with pytest.raises(capi.TsError) as e:
            b.add(case, ic)
        assert e.value.status == 4
        b.remove(ids[1])
        ids[1] = b.add(case, ic)
        b.run()
        outs = [b.get(i)[0] for i in ids]
    assert all(np.array_equal(o, outs[0]) for o in outs)


def test_batch_rejects_unbatchable(tslib):
    from turbostructred_gb300 import capi
    with capi.Batch(BUDGET) as b:
        c3 = capi.make_case(ndims=3, nx=8, ny=8, nz=8)
        with pytest.raises(capi.TsError) as e:
            b.add(c3, np.ones((8, 8, 8, 5)))
        assert e.value.status == 2
        with pytest.raises(capi.TsError) as e:
            b.get(12345)
        assert e.value.status == 8
        with pytest.raises(capi.TsError):
            b.set_tile(2, 24, 8)


def test_batch_unhealthy_problem_is_stopped(tslib):
    """A problem with a negative density is stopped with its health flag; the
    others are untouched."""
    from turbostructred_gb300 import capi
    probs = mixed_problems()[:3]
    bad_case, bad = probs[1][0], probs[1][1].copy()
    bad[0, 0, 100, 0] = -1.0
    res = run_batch([probs[0], (bad_case, bad), probs[2]])
    assert res[1][1]["health"] & capi.HEALTH_NEG_DENSITY
    ref = run_batch([probs[0], probs[2]])
    assert np.array_equal(res[0][0], ref[0][0]) and np.array_equal(res[2][0], ref[1][0])


@pytest.mark.parametrize("tile", [(1, 128, 1, 0), (1, 512, 1, 2), (2, 68, 1, 0), (2, 260, 1, 1), (2, 0, 1, 2)])
def test_batch_tiles_agree(tile, tslib):
    probs = mixed_problems(max_time=1e30, max_iter=15)
    base = run_batch(probs)
    other = run_batch(probs, tile=tile)
    for (a, ai), (b, bi) in zip(base, other):
        assert ai["iteration"] == bi["iteration"]
        assert relmax(b, a) <= 1e-5


def test_batch_autotune_restores_state(tslib):
    from turbostructred_gb300 import capi
    probs = mixed_problems(max_time=1e30, max_iter=20)
    base = run_batch(probs)
    with capi.Batch(BUDGET) as b:
        ids = [b.add(c, v) for c, v in probs]
        b.step(5)
        st0 = b.stats()
        tx, ty, ct = b.autotune(4)
        assert tx in (0, 260, 132, 68) and ty == 1
        assert b.stats()["stages"] == st0["stages"]
        assert all(b.get(i, want_state=False)[1]["iteration"] == 5 for i in ids)
        b.run()
        got = [b.get(i) for i in ids]
    for (g, gi), (r, ri) in zip(got, base):
        assert gi["iteration"] == 20
        assert relmax(g, r) <= 1e-5


def test_batch_admission_and_retirement_beside_queued_stages(tslib):
    """Problems added, read back and removed while stages are queued (the
    served loop's pattern: ts_batch_launch, uploads and read-backs, then
    ts_batch_wait) give the same results as the problems alone, bit for bit;
    a removed problem's slot is not reused before the queued stages drain."""
    from turbostructred_gb300 import capi
    probs = mixed_problems()
    alone = [run_batch([p])[0] for p in probs]
    results = {}
    with capi.Batch(BUDGET) as b:
        owner = {}
        pending = list(range(len(probs)))
        for _ in range(2):
            k = pending.pop(0)
            owner[b.add(*probs[k])] = k
        finished = []
        while owner:
            b.launch(5)
            # beside the queued stages: admit one, retire what finished earlier
            if pending:
                k = pending.pop(0)
                owner[b.add(*probs[k])] = k
            for pid in finished:
                results[owner.pop(pid)] = b.get(pid)
                b.remove(pid)
            b.wait()
            finished = b.finished()
    for k in range(len(probs)):
        assert results[k][1]["iteration"] == alone[k][1]["iteration"]
        assert np.array_equal(results[k][0], alone[k][0]), k


def tail_tubes():
    """1D problems that end in the batch's tail mode: sizes up to 16 clusters'
    worth of cells, PWC/limited/ENO2, Roe/HLLC, stiffened gas, periodic."""
    from turbostructred_gb300 import capi
    tube = [0.5, 1.0, 0.0, 1.0, 0.125, 0.0, 0.1]
    stiff = [0.5, 1.5, 0.2, 4.0, 0.8, -0.3, 0.5]
    specs = [
        (dict(ndims=1, nx=4096, periodic=(0, 1, 1), recon=3, solver=1, cfl=0.5, bc=[NAT] * 6), tube, 0.05),
        (dict(ndims=1, nx=1531, periodic=(0, 1, 1), recon=0, solver=3, cfl=0.5, bc=[NAT] * 6), tube, 0.08),
        (dict(ndims=1, nx=2000, periodic=(0, 1, 1), recon=3, solver=1, gamma=4.4, eos=1, p_inf=6.0, cfl=0.5,
              bc=[NAT] * 6), stiff, 0.01),
        (dict(ndims=1, nx=777, periodic=(1, 1, 1), recon=2, solver=3, cfl=0.4), tube, 0.05),
        (dict(ndims=1, nx=8128, periodic=(0, 1, 1), recon=3, limiter=1, solver=1, cfl=0.5, bc=[SYM] * 6), tube,
         0.004),
        (dict(ndims=1, nx=508, periodic=(0, 1, 1), recon=0, solver=1, cfl=0.5, bc=[NAT] * 6), tube, 0.1),
        (dict(ndims=1, nx=1017, periodic=(0, 1, 1), recon=3, solver=3, cfl=0.45, external_force=(0.3, 0.0, 0.0),
              uniform_acceleration=(-0.2, 0.0, 0.0), bc=[INLET, WALL] + [NAT] * 4), tube, 0.05),
        (dict(ndims=1, nx=300, periodic=(0, 1, 1), recon=3, solver=1, cfl=0.5,
              bc=[(2, 0.0, (0.2, 0.0, 0.0), 0.0), (4, 0.0, (0.0, 0.0, 0.0), 0.0)] + [NAT] * 4), tube, 0.08),
    ]
    out = []
    for n, (kw, params, t_end) in enumerate(specs):
        case = capi.make_case(**dict(kw, max_time=t_end, max_iter=100000))
        out.append((case, capi.fill_scenario(case, 0, 31 + n, params)))
    return out


@pytest.mark.parametrize("limits", ["t_end", "max_iter_and_snapshots"])
def test_batch_tail_mode_equals_stage_path(limits, tslib):
    """The cluster tail kernel (state on chip, many stages per launch) gives
    the stage-by-stage result bit for bit, in far fewer launches, with the
    Run loop's end conditions and SaveSolutionTime's dt clipping."""
    from turbostructred_gb300 import capi
    probs = tail_tubes()
    if limits != "t_end":
        probs = [(dict(c, max_time=1e30, max_iter=37 + 11 * k, save_solution_time=c["max_time"] / 7), v)
                 for k, (c, v) in enumerate(probs)]
    res, launches = {}, {}
    for tail in (True, False):
        with capi.Batch(BUDGET) as b:
            b.set_tail(tail)
            ids = [b.add(c, v) for c, v in probs]
            assert b.run() == 0
            res[tail] = [b.get(i) for i in ids]
            launches[tail] = b.stats()["launches"]
    for (got, info), (ref, rinfo) in zip(res[True], res[False]):
        assert info["iteration"] == rinfo["iteration"]
        assert info["time"] == rinfo["time"] and info["dt"] == rinfo["dt"]
        assert info["health"] == rinfo["health"] == 0
        assert np.array_equal(got, ref)
    assert launches[True] < launches[False] / 4


def test_c4_full_batch_sampled_against_fp64_oracle(tslib, oracle_mod):
    """The 4096-tube workload at full size: every tube finishes (or is stopped
    unhealthy), and sampled small tubes agree with the FP64 oracle run to the
    same end time within the mixed-precision bar."""
    from oracle import oracle as O
    from turbostructred_gb300 import capi, workloads
    probs = workloads.tubes(4096, seed=4096)
    budget = int(1.5 * sum(capi.batch_problem_bytes(c) for c, _ in probs)) + (64 << 20)
    with capi.Batch(budget) as b:
        ids = [b.add(c, v) for c, v in probs]
        assert b.run() == 0
        res = [b.get(i) for i in ids]
    healthy = [k for k, (_, info) in enumerate(res) if info["health"] == 0]
    assert len(healthy) >= 4000
    sample = [k for k in healthy if probs[k][0]["nx"] < 200][::7][:8]
    assert len(sample) >= 4
    for k in sample:
        case, ic = probs[k]
        got, info = res[k]
        ref, rinfo = oracle_mod.advance(case, O.embed(case, ic), -1)
        assert info["iteration"] == rinfo["iteration"], k
        ref_i = ref[0, 0, 1:-1].reshape(got.shape)
        assert l1(got, ref_i, 0) <= RHO_L1, (k, l1(got, ref_i, 0))
