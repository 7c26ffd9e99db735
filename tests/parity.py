"""Force-comparison measures shared by the GPU parity tests.

Two measures of an FP32 GPU force F against the FP64 oracle's F_ref:
  * normwise:  max_i |F_i - F_ref,i|_inf / max_i |F_ref,i|_inf;
  * per atom:  |F_i - F_ref,i|_2 / |F_ref,i|_2 over the atoms whose force
    magnitude is at least PER_ATOM_FLOOR x the largest magnitude of the
    system (below that floor an atom's force is a near-cancellation of much
    larger contributions, and its relative error measures that cancellation,
    not the kernels).
"""
import numpy as np

FORCE_TOL = 1e-5        # normwise, the 1e-5 relative target
PER_ATOM_TOL = 1e-5     # per atom, above the floor
PER_ATOM_FLOOR = 0.10   # fraction of the largest force magnitude


def nrel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def per_atom(f, ref, floor=PER_ATOM_FLOOR):
    """(median, max, atoms checked, atoms in total) of the per-atom relative error."""
    f = np.asarray(f, np.float64).reshape(-1, 3)
    ref = np.asarray(ref, np.float64).reshape(-1, 3)
    mag = np.linalg.norm(ref, axis=1)
    sel = mag >= floor * mag.max()
    if not np.any(sel):
        return 0.0, 0.0, 0, len(mag)
    rel = np.linalg.norm(f - ref, axis=1)[sel] / mag[sel]
    return float(np.median(rel)), float(rel.max()), int(sel.sum()), len(mag)


def check_force(f, ref, label, tol=FORCE_TOL, atom_tol=PER_ATOM_TOL, floor=PER_ATOM_FLOOR):
    """Asserts both measures and prints them; returns (normwise, per-atom max)."""
    n = nrel(f, ref)
    med, mx, k, tot = per_atom(f, ref, floor)
    print(f"{label}: normwise {n:.2e}; per atom (|F| >= {floor:g} max, {k}/{tot} atoms) "
          f"median {med:.2e} max {mx:.2e}")
    assert n < tol, (label, "normwise", n)
    assert mx < atom_tol, (label, "per atom", mx)
    return n, mx
