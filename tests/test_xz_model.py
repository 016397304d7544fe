"""CPU: the x / z pass model (tests/xz_model.py).  Its tableau equals the
oracle's after every instruction; the blocked form -- the rank-1 updates of
consecutive random measurements deferred and applied in one pass -- gives
the same trace records and final state as one measurement at a time, for
every block size; so does the cluster pass's decomposition."""
import numpy as np
import pytest

from sdim_gb300 import workloads
from tests.conftest import oracle_run
from tests.xz_model import blocked_xz, cluster_xz, sequential_xz


def _ops(spec):
    return [(int(g), int(q), int(t)) for g, q, t, _ in spec.op_table()]


def _spec(n, d, seed, kind):
    if kind == "hpc":
        return workloads.random_hpc(n, d, 4 * n + 8, seed=seed, mr_every=max(1, 2 * n), mr_fraction=0.3)
    # measure everything twice, with Paulis between: a random sweep, then a deterministic one
    base = workloads.random_hpc(n, d, 4 * n + 8, seed=seed)
    rng = np.random.default_rng(seed)
    ops = list(base.ops)
    ops += [(("X", "Z", "X_INV", "Z_INV")[int(rng.integers(4))], int(q), None, {}) for q in rng.integers(n, size=n)]
    ops += [("RESET" if rng.random() < 0.3 else "M", q, None, {}) for q in range(n)]
    return workloads.CircuitSpec(n, d, ops, f"twice_n{n}_d{d}")


def _oracle_xz(spec, n):
    snaps = oracle_run([spec], 0, 0, 1, noise=False, snapshots=True)["snapshots"].astype(np.int64)
    nn = n * n
    x, z = snaps[:, :nn].reshape(-1, n, n), snaps[:, nn:2 * nn].reshape(-1, n, n)
    dx, dz = snaps[:, 2 * nn + n:3 * nn + n].reshape(-1, n, n), snaps[:, 3 * nn + n:4 * nn + n].reshape(-1, n, n)
    return np.concatenate([x, dx], axis=2), np.concatenate([z, dz], axis=2)


@pytest.mark.parametrize("d", [3, 5, 7])
@pytest.mark.parametrize("n,kind", [(1, "hpc"), (4, "twice"), (9, "hpc"), (12, "twice")])
def test_model_tableau_matches_oracle(n, d, kind):
    spec = _spec(n, d, seed=10 * n + d, kind=kind)
    ops = _ops(spec)
    ox, oz = _oracle_xz(spec, n)
    for i in range(len(ops)):
        _, tab = sequential_xz(n, d, ops[:i + 1])
        assert np.array_equal(tab.X, ox[i]) and np.array_equal(tab.Z, oz[i]), (n, d, i, ops[i])


@pytest.mark.parametrize("block", [1, 2, 3, 6, 64])
@pytest.mark.parametrize("d", [3, 5, 7, 11])
@pytest.mark.parametrize("n,kind", [(1, "twice"), (2, "hpc"), (5, "twice"), (17, "hpc"), (40, "twice")])
def test_blocked_matches_sequential(n, d, kind, block):
    ops = _ops(_spec(n, d, seed=n * 31 + d, kind=kind))
    seq, st = sequential_xz(n, d, ops)
    blk, bt = blocked_xz(n, d, ops, block)
    assert len(seq) == len(blk)
    for i, ((h1, r1, z1), (h2, r2, z2)) in enumerate(zip(seq, blk)):
        assert h1 == h2, (i, h1, h2)
        assert np.array_equal(r1, r2), i
        assert (z1 is None) == (z2 is None) and (z1 is None or np.array_equal(z1, z2)), i
    assert np.array_equal(st.X, bt.X) and np.array_equal(st.Z, bt.Z) and np.array_equal(st.C, bt.C)


def test_blocked_sweeps_are_mostly_random():
    """The final MEASURE sweep of a random circuit is where the blocks pay:
    nearly all its outcomes are random, so nearly every measurement joins a
    block."""
    n, d = 40, 5
    recs, _ = sequential_xz(n, d, _ops(workloads.random_hpc(n, d, 8 * n, seed=3)))
    kinds = [h[0] for h, _, _ in recs]
    assert kinds.count("rand") >= 0.8 * n


@pytest.mark.parametrize("d", [3, 5, 7])
@pytest.mark.parametrize("n,kind", [(1, "twice"), (3, "hpc"), (6, "twice"), (13, "hpc"), (30, "twice"), (37, "hpc")])
def test_cluster_decomposition_matches_sequential(n, d, kind):
    """The cluster pass's arithmetic (slices, the unexponentiated pivot
    column with scaled factors, the deterministic slice sums as byte dot
    products and the cross-slice header term) gives the one-at-a-time
    records and final state; slices are empty for n < 4 and ragged when 4
    does not divide n."""
    ops = _ops(_spec(n, d, seed=n * 7 + d, kind=kind))
    seq, st = sequential_xz(n, d, ops)
    cl, ct = cluster_xz(n, d, ops)
    assert len(seq) == len(cl)
    for i, ((h1, r1, z1), (h2, r2, z2)) in enumerate(zip(seq, cl)):
        assert h1 == h2, (i, h1, h2)
        assert np.array_equal(r1, r2), i
        assert (z1 is None) == (z2 is None) and (z1 is None or np.array_equal(z1, z2)), i
    assert np.array_equal(st.X, ct.X) and np.array_equal(st.Z, ct.Z) and np.array_equal(st.C, ct.C)
    assert any(h[0] == "det" for h, _, _ in seq) or n == 1 or kind == "hpc"
