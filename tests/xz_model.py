"""CPU model of the odd-d trace engine's x / z pass (test infrastructure).

``sequential_xz`` restates what the x / z pass kernels do
(sdim_gb300/csrc/trace_u8.cuh, trace_split_u8.cuh, trace_cluster_u8.cuh)
over whole arrays: the tableau X, Z (rows = qudits, columns = the n
stabilizers then the n destabilizers), the common phase vector C, and per
measurement the trace record the phase pass replays -- the header (kind,
pivot, exponent, deterministic phase) and the factor row f over all 2n
generators, plus the z_q row after a RESET.  Its X and Z equal the
reference's tableau (sdim/tableau/tableau_prime.py:88-380) at every
instruction, checked against the oracle in tests/test_xz_model.py.

``cluster_xz`` restates the cluster pass's decomposition (candidates per
slice, the unexponentiated pivot column with scaled factors, deterministic
slice sums as byte dot products, the cross-slice header term) and gives the
same records and final state.

``blocked_xz`` computes the same records and the same final state with the
rank-1 updates of up to ``block`` consecutive random measurements deferred
and applied in one pass over the tableau: the form that reads and writes a
streamed tableau once per block instead of once per measurement.  Per
measurement it only touches rows (row q of X from the deferred updates) and
the few pivot columns, which it keeps explicit:
- row q:      x_q[g] = X0[q, g] + sum_h f_h[g] cx_h[q] for deferred columns;
- pivot p:    its column replayed through the deferred updates, then
              exponentiated; the destabilizer n + p and stabilizer p are
              then replaced and stay explicit until the flush;
- the flush:  X[:, g] = X0[:, g] + sum_h f_h[g] cx_h (Z likewise), and the
              phase dots DOT_h[g] = Z0[:, g] . cx_h + sum_{h' < h} f_h'[g]
              (cz_h' . cx_h), so one pass over Z0 serves every deferred
              measurement.
A deterministic outcome flushes first and is evaluated on the full tableau.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

H, H_INV, P, P_INV, CNOT, CNOT_INV = 5, 6, 7, 8, 9, 10
X_, X_INV, Z_, Z_INV = 1, 2, 3, 4
M, RESET = 14, 16


def _inv(x, d):
    return pow(int(x), d - 2, d)


class _Tab:
    def __init__(self, n, d):
        self.n, self.d = n, d
        self.X = np.zeros((n, 2 * n), dtype=np.int64)
        self.Z = np.zeros((n, 2 * n), dtype=np.int64)
        self.C = np.zeros(2 * n, dtype=np.int64)
        for k in range(n):
            self.Z[k, k] = 1          # stabilizer k = Z_k
            self.X[k, n + k] = 1      # destabilizer k = X_k

    def gate(self, gid, q, t):
        d, X, Z, C = self.d, self.X, self.Z, self.C
        if gid == H:
            x, z = X[q].copy(), Z[q].copy()
            nx = (-z) % d
            C[:] = (C + nx * x) % d
            X[q], Z[q] = nx, x
        elif gid == H_INV:
            x, z = X[q].copy(), Z[q].copy()
            nz = (-x) % d
            C[:] = (C + z * nz) % d
            X[q], Z[q] = z, nz
        elif gid in (P, P_INV):
            x = X[q]
            tt = ((x * (x - 1)) // 2) % d
            if gid == P:
                C[:] = (C + tt) % d
                Z[q] = (Z[q] + x) % d
            else:
                C[:] = (C + d - tt) % d
                Z[q] = (Z[q] + d - x) % d
        elif gid in (CNOT, CNOT_INV):
            if gid == CNOT:
                X[t] = (X[t] + X[q]) % d
                Z[q] = (Z[q] + d - Z[t]) % d
            else:
                X[t] = (X[t] + d - X[q]) % d
                Z[q] = (Z[q] + Z[t]) % d
        elif gid in (X_, X_INV, Z_, Z_INV):
            cz = {X_: d - 1, X_INV: 1, Z_: 0, Z_INV: 0}[gid]
            cx = {X_: 0, X_INV: 0, Z_: 1, Z_INV: d - 1}[gid]
            C[:] = (C + cz * Z[q] + cx * X[q]) % d
        else:
            raise ValueError(f"gate id {gid} is not modelled")

    # -- one measurement on the full tableau
    def deterministic(self, q):
        n, d, X, Z, C = self.n, self.d, self.X, self.Z, self.C
        f = X[q, n:].copy()
        P_ = int((f * C[:n]).sum()) % d
        cd = (X[:, :n] * Z[:, :n]).sum(axis=0) % d
        Dd = int(((cd * ((f * (f - 1)) // 2)) % d).sum()) % d
        # T = sum_k sum_{i < j} f_i z_k[i] f_j x_k[j]
        fz = (Z[:, :n] * f) % d
        pre = (np.cumsum(fz, axis=1) - fz) % d
        T = int(((pre * ((X[:, :n] * f) % d)) % d).sum()) % d
        aphc = (P_ + T + Dd) % d
        row = np.zeros(2 * n, dtype=np.int64)
        row[:n] = f
        return ("det", 0, 1, aphc), row

    def random(self, q, p):
        n, d, X, Z, C = self.n, self.d, self.X, self.Z, self.C
        xv = int(X[q, p])
        ex = 1
        if xv != 1:
            ex = _inv(xv, d)
            s0 = int((X[:, p] * Z[:, p]).sum()) % d
            C[p] = (C[p] * ex + (s0 * ((ex * (ex - 1)) // 2 % d)) % d) % d
            X[:, p] = (X[:, p] * ex) % d
            Z[:, p] = (Z[:, p] * ex) % d
        cx, cz = X[:, p].copy(), Z[:, p].copy()
        s1 = int((cx * cz).sum()) % d
        phc = int(C[p])
        fw = (-X[q]) % d
        fw[p] = 0
        dot = (Z.T @ cx) % d
        X[:] = (X + np.outer(cx, fw)) % d
        Z[:] = (Z + np.outer(cz, fw)) % d
        half = (s1 * ((fw * (fw - 1)) // 2)) % d
        C[:] = np.where(fw != 0, (C + phc * fw + (fw * dot) % d + half) % d, C)
        X[:, n + p], Z[:, n + p], C[n + p] = cx, cz, phc
        X[:, p], Z[:, p], C[p] = 0, 0, 0
        Z[q, p] = 1
        return ("rand", p, ex, 0), fw


def _records_append(recs, hdr, row, reset_row):
    recs.append((hdr, row.copy(), None if reset_row is None else reset_row.copy()))


def sequential_xz(n: int, d: int, ops) -> Tuple[List, _Tab]:
    """ops: rows (gate id, qudit, target).  Returns (records, tableau)."""
    tab = _Tab(n, d)
    recs: List = []
    for gid, q, t in ops:
        if gid in (M, RESET):
            stab = np.nonzero(tab.X[q, :n])[0]
            hdr, row = tab.deterministic(q) if len(stab) == 0 else tab.random(q, int(stab[0]))
            _records_append(recs, hdr, row, tab.Z[q].copy() if gid == RESET else None)
        else:
            tab.gate(gid, q, t)
    return recs, tab


class _Deferred:
    """The block's deferred rank-1 updates over the state (X0, Z0, C0) at its start."""

    def __init__(self, tab: _Tab):
        self.tab = tab
        self.fw: List[np.ndarray] = []
        self.cx: List[np.ndarray] = []
        self.cz: List[np.ndarray] = []
        self.phc: List[int] = []
        self.s1: List[int] = []
        self.explicit: Dict[int, List] = {}  # column -> [x, z, c], current values

    def __len__(self):
        return len(self.fw)

    def _replay(self, g):
        """Column g brought through every deferred update (data and phase)."""
        d, tab = self.tab.d, self.tab
        x, z, c = tab.X[:, g].copy(), tab.Z[:, g].copy(), int(tab.C[g])
        for fw, cx, cz, phc, s1 in zip(self.fw, self.cx, self.cz, self.phc, self.s1):
            f = int(fw[g])
            if f:
                dot = int((z * cx).sum()) % d
                c = (c + phc * f + (f * dot) % d + (s1 * ((f * (f - 1)) // 2)) % d) % d
                x, z = (x + f * cx) % d, (z + f * cz) % d
        return [x, z, c]

    def column(self, g):
        if g not in self.explicit:
            self.explicit[g] = self._replay(g)
        return self.explicit[g]

    def row(self, blk, q):
        """Row q of X or Z (blk 'x' / 'z') over all 2n generators, current."""
        d, tab = self.tab.d, self.tab
        base = (tab.X if blk == "x" else tab.Z)[q].copy()
        for fw, cx, cz in zip(self.fw, self.cx, self.cz):
            base = (base + fw * (cx[q] if blk == "x" else cz[q])) % d
        for g, (x, z, _) in self.explicit.items():
            base[g] = (x if blk == "x" else z)[q]
        return base

    def random(self, q, p, rowx):
        n, d = self.tab.n, self.tab.d
        col = self.column(p)
        xv = int(rowx[p])
        ex = 1
        if xv != 1:
            ex = _inv(xv, d)
            s0 = int((col[0] * col[1]).sum()) % d
            col[2] = (col[2] * ex + (s0 * ((ex * (ex - 1)) // 2 % d)) % d) % d
            col[0], col[1] = (col[0] * ex) % d, (col[1] * ex) % d
        cx, cz = col[0].copy(), col[1].copy()
        s1 = int((cx * cz).sum()) % d
        phc = int(col[2])
        fw = (-rowx) % d
        fw[p] = 0
        # explicit columns take this update now, the others at the flush
        for g, e in self.explicit.items():
            f = int(fw[g])
            if f:
                dot = int((e[1] * cx).sum()) % d
                e[2] = (e[2] + phc * f + (f * dot) % d + (s1 * ((f * (f - 1)) // 2)) % d) % d
                e[0], e[1] = (e[0] + f * cx) % d, (e[1] + f * cz) % d
        self.fw.append(fw)
        self.cx.append(cx)
        self.cz.append(cz)
        self.phc.append(phc)
        self.s1.append(s1)
        zq = np.zeros(n, dtype=np.int64)
        zq[q] = 1
        self.explicit[n + p] = [cx, cz, phc]
        self.explicit[p] = [np.zeros(n, dtype=np.int64), zq, 0]
        return ("rand", p, ex, 0), fw

    def flush(self):
        """One pass over every deferred column, then the explicit ones."""
        tab, d = self.tab, self.tab.d
        k = len(self.fw)
        if k:
            F = np.stack(self.fw)                      # (k, 2n)
            CX, CZ = np.stack(self.cx), np.stack(self.cz)  # (k, n)
            G = (CZ @ CX.T) % d                        # G[h', h] = cz_h' . cx_h
            D0 = (CX @ tab.Z) % d                      # D0[h, g] = Z0[:, g] . cx_h
            C = tab.C.copy()
            for h in range(k):
                f = F[h]
                dot = (D0[h] + (F[:h] * G[:h, h][:, None]).sum(axis=0)) % d
                half = (self.s1[h] * ((f * (f - 1)) // 2)) % d
                C = np.where(f != 0, (C + self.phc[h] * f + (f * dot) % d + half) % d, C)
            tab.X[:] = (tab.X + CX.T @ F) % d
            tab.Z[:] = (tab.Z + CZ.T @ F) % d
            tab.C[:] = C
        for g, (x, z, c) in self.explicit.items():
            tab.X[:, g], tab.Z[:, g], tab.C[g] = x, z, c
        self.__init__(tab)


def blocked_xz(n: int, d: int, ops, block: int) -> Tuple[List, _Tab]:
    """sequential_xz with up to `block` random measurements deferred."""
    tab = _Tab(n, d)
    dfr = _Deferred(tab)
    recs: List = []
    for gid, q, t in ops:
        if gid in (M, RESET):
            rowx = dfr.row("x", q)
            stab = np.nonzero(rowx[:n])[0]
            if len(stab) == 0:
                dfr.flush()
                hdr, row = tab.deterministic(q)
            else:
                if len(dfr) == block:
                    dfr.flush()
                    rowx = dfr.row("x", q)
                hdr, row = dfr.random(q, int(stab[0]), rowx)
            _records_append(recs, hdr, row, dfr.row("z", q) if gid == RESET else None)
        else:
            dfr.flush()
            tab.gate(gid, q, t)
    dfr.flush()
    return recs, tab


def _byte_dot(a, b):
    """dp4a over one word: the sum of four byte products."""
    return int((np.asarray(a, dtype=np.int64) * np.asarray(b, dtype=np.int64)).sum())


def cluster_xz(n: int, d: int, ops, K: int = 8) -> Tuple[List, _Tab]:
    """The arithmetic of the cluster x / z pass (sdim_gb300/csrc/
    trace_cluster_u8.cuh) over whole arrays: H = K / 2 stabilizer slices of
    C0 = ceil(n / H) columns.
    - Pivot: each slice's lowest column with x_q != 0 is its candidate, the
      lowest candidate the pivot.
    - Random outcome: the rank-1 update runs with the pivot column as it
      stands and the factors scaled by the exponent e (x += (e f) cx is the
      update with the exponentiated column e cx); the dots and the column's
      self-dot are taken on the unexponentiated column and scaled by e, e^2.
    - Deterministic outcome: per slice the partial sums P_c = sum f c and, per
      row, words of four columns with Z_w = f . z, X_w = f . x and the in-word
      terms sum_j x_j (z . G_j), G_j holding f_i f_j in byte i < j and
      f_j (f_j - 1) / 2 in byte j (so the in-slice cross terms and the
      f (f - 1) / 2 x.z terms share one sum, phi = 1 for odd d); the header
      pass adds the cross-slice term sum_k sum_{c' < c} Z_c'[k] X_c[k].
    Returns (records, tableau) as sequential_xz does."""
    assert d % 2 == 1
    tab = _Tab(n, d)
    X, Z, C = tab.X, tab.Z, tab.C
    H = K // 2
    C0 = -(-n // H)
    slices = [(c * C0, max(c * C0, min(n, (c + 1) * C0))) for c in range(H)]  # empty past n
    recs: List = []
    for gid, q, t in ops:
        if gid not in (M, RESET):
            tab.gate(gid, q, t)
            continue
        cands = [a + int(np.nonzero(X[q, a:b])[0][0]) for a, b in slices if b > a and X[q, a:b].any()]
        if cands:
            p = min(cands)
            cx, cz = X[:, p].copy(), Z[:, p].copy()  # unexponentiated
            xv = int(X[q, p])
            e = 1 if xv == 1 else _inv(xv, d)
            f = (-X[q]) % d
            f[p] = 0
            g = (e * f) % d
            dot_raw = (Z.T @ cx) % d  # old z
            X[:] = (X + np.outer(cx, g)) % d
            Z[:] = (Z + np.outer(cz, g)) % d
            s0 = int((cx * cz).sum()) % d
            s1 = (e * e % d) * s0 % d
            phc = int(C[p]) if e == 1 else (int(C[p]) * e + (s0 * ((e * (e - 1) // 2) % d)) % d) % d
            dot = (e * dot_raw) % d
            half = (s1 * ((f * (f - 1)) // 2)) % d
            C[:] = np.where(f != 0, (C + phc * f + (f * dot) % d + half) % d, C)
            X[:, n + p], Z[:, n + p], C[n + p] = (e * cx) % d, (e * cz) % d, phc
            X[:, p], Z[:, p], C[p] = 0, 0, 0
            Z[q, p] = 1
            hdr, row = ("rand", p, e, 0), f
        else:
            fall = X[q, n:].copy()
            P_, A = 0, 0
            zc, xc = [], []
            for a, b in slices:
                f = np.zeros(4 * -(-(b - a) // 4), dtype=np.int64)
                f[:b - a] = fall[a:b]
                P_ += int((fall[a:b] * C[a:b]).sum())
                G = []
                for w in range(len(f) // 4):
                    fw = f[4 * w:4 * w + 4]
                    G.append([[fw[i] * fw[j] if i < j else (fw[j] * (fw[j] - 1)) // 2 if i == j else 0
                               for i in range(4)] for j in range(4)])
                zk, xk = np.zeros(n, dtype=np.int64), np.zeros(n, dtype=np.int64)
                for k in range(n):
                    xr = np.zeros(len(f), dtype=np.int64)
                    zr = np.zeros(len(f), dtype=np.int64)
                    xr[:b - a], zr[:b - a] = X[k, a:b], Z[k, a:b]
                    pre = acc = xs = 0
                    for w in range(len(f) // 4):
                        fw, xw, zw = f[4 * w:4 * w + 4], xr[4 * w:4 * w + 4], zr[4 * w:4 * w + 4]
                        if not fw.any():
                            continue
                        zs, xsw = _byte_dot(zw, fw), _byte_dot(xw, fw)
                        inw = sum(int(xw[j]) * _byte_dot(zw, G[w][j]) for j in range(4))
                        acc = (acc + pre * xsw + inw) % d
                        pre = (pre + zs) % d
                        xs += xsw
                    zk[k], xk[k] = pre, xs % d
                    A += acc
                zc.append(zk)
                xc.append(xk)
            cross = 0
            zb = np.zeros(n, dtype=np.int64)
            for c in range(H):
                cross += int((zb * xc[c]).sum())
                zb += zc[c]
            aphc = (P_ + A + cross) % d
            row = np.zeros(2 * n, dtype=np.int64)
            row[:n] = fall
            hdr = ("det", 0, 1, aphc)
        _records_append(recs, hdr, row, Z[q].copy() if gid == RESET else None)
    return recs, tab
