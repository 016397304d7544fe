"""GPU: batched persistent launches over uneven programs equal per-program
runs and the oracle; a program's records do not depend on what else runs in
the same batch."""
import numpy as np
import pytest

from sdim_gb300 import workloads
from sdim_gb300.batch import BatchRunner
from tests.conftest import oracle_run

pytestmark = pytest.mark.gpu


def _small_uneven(count=48, seed=3, n_max=300):
    return workloads.uneven_batch(count, seed=seed, n_max=n_max, shots_max=8)


def test_uneven_batch_matches_oracle():
    items = _small_uneven()
    br = BatchRunner()
    for it in items:
        br.add_spec(it.spec, it.shots, it.seed)
    outs = br.run()
    for it, out in zip(items, outs):
        ref = oracle_run([it.spec], it.seed, 0, it.shots)["records"]
        assert np.array_equal(out, ref), it.spec.name


def test_batch_result_independent_of_mix_and_plain_form():
    items = _small_uneven(24, seed=8)
    br = BatchRunner()
    for it in items:
        br.add_spec(it.spec, it.shots, it.seed)
    mixed = br.run()
    plain = br.run(plain=True)
    for a, b in zip(mixed, plain):
        assert np.array_equal(a, b)
    for k in (0, 5, 17):
        alone = BatchRunner()
        alone.add_spec(items[k].spec, items[k].shots, items[k].seed)
        assert np.array_equal(alone.run()[0], mixed[k])


def test_uneven_batch_with_large_programs():
    # n >= 520 puts every dimension's tableau in global-memory slots
    items = workloads.uneven_batch(8, seed=11, n_min=520, n_max=640, shots_max=2)
    br = BatchRunner()
    for it in items:
        br.add_spec(it.spec, it.shots, it.seed)
    outs = br.run()
    for it, out in list(zip(items, outs))[:2]:
        ref = oracle_run([it.spec], it.seed, 0, it.shots)["records"]
        assert np.array_equal(out, ref), it.spec.name
