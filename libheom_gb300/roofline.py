"""Algorithmic traffic and work of the fused stage kernels.

Bytes: every vector a stage launch must read or write for its own elements,
each counted once (neighbour-ADO reads of the right-hand-side input are cache
hits; buffers that alias in FP64 mode count once).  State vectors are FP64
complex (16 B); bulk vectors are 8 B in mixed precision and 16 B in FP64.

  rk4   s1: Y1 S | Y2 acc          s2,s3: Y S acc | Y' acc      s4: Y4 acc | S (Y1)
        (mixed: s2,s3 read the state's bulk copy Y1 instead of S)
  lsrk4 s:  Y S (buff) | buff S' (Y')        (buff is a bulk vector: FP32 in mixed)
  rkdp  s1..s6: Y S K_1..K_{s-1} | K_s Y'  (s6 writes S' and Y' instead of Y')
        s7: Y7 K_1..K_6 S' S | -           (mixed: the FP32 copies of S' and S)
Flops: real floating-point operations per element of the right-hand side as
evaluated by the diagonal-coupling kernel: the commutator (4 real FMA per term
for real H, 8 for complex H), the damping term, and 8 (+2 for the n_k scale)
per active +1 / -1 mode term.
"""
from __future__ import annotations

import numpy as np

STATE = 16


def _units(solver: str, mixed: bool):
    """List of (reads, writes) per launch; entries are ('S'|'B', name)."""
    B = 8 if mixed else 16
    sep = mixed

    def vec(kind, name):
        return (kind, name)

    if solver == "rk4":
        Y1 = vec("B", "Yb0") if sep else vec("S", "S")
        base = Y1 if sep else vec("S", "S")  # the stage input's base: the state's bulk copy in mixed
        stages = [
            ([Y1, vec("S", "S")], [vec("B", "Y2"), vec("S", "acc")]),
            ([vec("B", "Y2"), base, vec("S", "acc")], [vec("B", "Y3"), vec("S", "acc")]),
            ([vec("B", "Y3"), base, vec("S", "acc")], [vec("B", "Y4"), vec("S", "acc")]),
            ([vec("B", "Y4"), vec("S", "acc")], [vec("S", "S")] + ([vec("B", "Yb0")] if sep else [])),
        ]
    elif solver == "lsrk4":
        stages = []
        for s in range(4):
            i, o = s & 1, 1 - (s & 1)
            Yi = vec("B", f"Yb{i}") if sep else vec("S", f"S{i}")
            buff = vec("B" if sep else "S", "buff")  # FP32 in mixed precision
            reads = [Yi, vec("S", f"S{i}")] + ([buff] if s else [])
            writes = [buff, vec("S", f"S{o}")] + ([vec("B", f"Yb{o}")] if sep else [])
            stages.append((reads, writes))
    elif solver == "rkdp":
        stages = []
        Ycur = vec("B", "Ybc") if sep else vec("S", "Sc")
        for s in range(6):
            Yin = Ycur if s == 0 else vec("B", f"Y{s}")
            reads = [Yin, vec("S", "Sc")] + [vec("B", f"K{j}") for j in range(s)]
            writes = [vec("B", f"K{s}")]
            writes += [vec("B", f"Y{s + 1}")] if s < 5 else ([vec("S", "So")] + ([vec("B", "Ybo")] if sep else []))
            stages.append((reads, writes))
        Y7 = vec("B", "Ybo") if sep else vec("S", "So")
        # the error scale reads both states: their FP32 copies in mixed precision
        scale = [vec("B", "Ybo"), vec("B", "Ybc")] if sep else [vec("S", "So"), vec("S", "Sc")]
        stages.append(([Y7] + [vec("B", f"K{j}") for j in range(6)] + scale, []))
    else:
        raise ValueError(solver)
    out = []
    for reads, writes in stages:
        seen = set()
        nb = 0
        for kind, name in reads:
            if name in seen:
                continue
            seen.add(name)
            nb += STATE if kind == "S" else B
        for kind, name in writes:
            nb += STATE if kind == "S" else B
        out.append(nb)
    return out


def bytes_per_element(solver: str, mixed: bool):
    """(bytes per element per step/attempt, launches per step/attempt)."""
    per = _units(solver, mixed)
    return sum(per), len(per)


def active_terms(p):
    """Counts of nonzero +1 and -1 coefficients summed over elements (diagonal V)."""
    n = p.n_level
    plus = minus = 0
    for u in range(p.n_noise):
        v = np.diag(p.V[u])
        cphi = 1j * (v[:, None] - v[None, :])
        cpsi = v[:, None] + v[None, :]
        sv = p.S[u] @ p.phi_0[u]
        av = p.A[u] @ p.phi_0[u]
        for k in range(len(p.sigma[u])):
            plus += int(np.count_nonzero(cphi * p.sigma[u][k]))
            minus += int(np.count_nonzero(cphi * sv[k] - cpsi * av[k]))
    return plus, minus


def flops_per_element(p) -> float:
    n = p.n_level
    h_real = bool(np.all(np.imag(p.H) == 0))
    comm = n * (8 if h_real else 16)
    plus, minus = active_terms(p)
    n2 = n * n
    return comm + 8 + (8 * plus + 10 * minus) / n2
