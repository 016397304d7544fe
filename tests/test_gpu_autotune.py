"""GPU: the autotuner times every route on the device, keeps the fastest, and
the tuned run gives the same records as the default route and the oracle.
Also the shot-group team overrides on the far side of the library's own
choice (a warp per group at n >= 160, a CTA per group below), which only
the tuner selects."""
import numpy as np
import pytest

from sdim_gb300 import Program, _lib, autotune, workloads
from sdim_gb300.batch import BatchRunner
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("d,n,shots", [(2, 17, 256), (3, 40, 100), (5, 230, 64)])
def test_tuned_program_matches_default_and_oracle(cuda_ctx, d, n, shots):
    if d == 2:
        spec = workloads.surface_memory(3, 2, prob=0.03)
    else:
        spec = workloads.random_hpc(n, d, 4 * n, seed=n + d, mr_every=n, mr_fraction=0.1)
    prog = Program(spec.build())
    dp = prog.compile()
    tuner = autotune.Autotuner(ctx=cuda_ctx, reps=1)
    res = tuner.tune_program(dp, shots, seed=3)
    cands = autotune.program_candidates(dp.enc.d, dp.enc.n, shots, cuda_ctx.smem_optin, cuda_ctx.num_sms)
    assert res.best in cands
    assert set(res.times_ms) == {c.name for c in cands}
    assert tuner.flags_for_program(dp, shots) == res.best.flags
    out = np.empty((shots, dp.num_records), dtype=np.uint8)
    rc = cuda_ctx.lib.sdim_run(cuda_ctx.ptr, dp.ptr, 3, 0, shots, out.ctypes.data, res.best.flags)
    _lib.check(rc, cuda_ctx.ptr)
    assert np.array_equal(out, prog.sample(shots, seed=3))
    assert np.array_equal(out[:4], oracle_run([spec], 3, 0, 4)["records"])
    # the drop-in's tuned engine
    assert np.array_equal(prog.sample(shots, seed=3, engine="tuned"), out)


@pytest.mark.parametrize("d,n,flag", [(2, 20, "cta"), (3, 24, "cta"), (5, 170, "warp"), (2, 170, "warp")])
def test_team_overrides_against_the_oracle(d, n, flag):
    spec = workloads.random_hpc(n, d, 3 * n, seed=7 * n + d, mr_every=n // 2, mr_fraction=0.2)
    prog = Program(spec.build())
    dp = prog.compile()
    ctx = prog.context
    out = np.empty((45, dp.num_records), dtype=np.uint8)
    f = _lib.FLAG_TEAM_CTA if flag == "cta" else _lib.FLAG_TEAM_WARP
    rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, 9, 2, 45, out.ctypes.data, f)
    _lib.check(rc, ctx.ptr)
    assert np.array_equal(out, oracle_run([spec], 9, 2, 45)["records"])
    assert np.array_equal(out, prog.sample(45, seed=9, shot0=2))


def test_tuned_batch_matches_default(cuda_ctx):
    runner = BatchRunner(cuda_ctx)
    rng = np.random.default_rng(5)
    for i in range(12):
        d = int(rng.choice([2, 3, 5, 7]))
        n = int(rng.integers(4, 200))
        spec = workloads.random_hpc(n, d, 4 * n, seed=i)
        runner.add_spec(spec, shots=int(rng.integers(1, 70)), seed=100 + i)
    base = runner.run()
    tuner = autotune.Autotuner(ctx=cuda_ctx, reps=1)
    res = tuner.tune_batch(runner)
    assert res.best in autotune.batch_candidates()
    tuned = runner.run(flags=tuner.flags_for_batch(runner))
    for a, b in zip(base, tuned):
        assert np.array_equal(a, b)
    for a, b in zip(base, runner.run(engine="tuned")):
        assert np.array_equal(a, b)
