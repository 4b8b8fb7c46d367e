"""Hamiltonians of the hot-path workloads, as (op, couplings) lists usable by the
oracle and by qsgpu.OperatorTerm."""
import numpy as np


def xxz(L, J=1.0, delta=0.5, periodic=True):
    bonds = [(i, i % L + 1) for i in range(1, L + 1)] if periodic else [(i, i + 1) for i in range(1, L)]
    return [("+-", [(J / 2, a, b) for a, b in bonds]),
            ("-+", [(J / 2, a, b) for a, b in bonds]),
            ("zz", [(J * delta, a, b) for a, b in bonds])]


def j1j2(L, J1=1.0, J2=0.5):
    b1 = [(i, i % L + 1) for i in range(1, L + 1)]
    b2 = [(i, (i + 1) % L + 1) for i in range(1, L + 1)]
    return [("+-", [(J1 / 2, a, b) for a, b in b1] + [(J2 / 2, a, b) for a, b in b2]),
            ("-+", [(J1 / 2, a, b) for a, b in b1] + [(J2 / 2, a, b) for a, b in b2]),
            ("zz", [(J1, a, b) for a, b in b1] + [(J2, a, b) for a, b in b2])]


def tfim(L, J=1.0, h=0.7):
    bonds = [(i, i % L + 1) for i in range(1, L + 1)]
    return [("zz", [(J, a, b) for a, b in bonds]), ("x", [(h, i) for i in range(1, L + 1)])]


def xyz_field(L, seed=0):
    """A Hermitian operator with y terms (complex) and fields, translation invariant."""
    bonds = [(i, i % L + 1) for i in range(1, L + 1)]
    return [("xx", [(0.3, a, b) for a, b in bonds]), ("yy", [(0.45, a, b) for a, b in bonds]),
            ("zz", [(0.8, a, b) for a, b in bonds]), ("y", [(0.2, i) for i in range(1, L + 1)]),
            ("z", [(0.1, i) for i in range(1, L + 1)])]


def to_terms(qs, spec):
    return [qs.OperatorTerm(op, c) for op, c in spec]


def seeded(n, seed=20261203, complex_=False):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(n)
    if complex_:
        v = v + 1j * rng.standard_normal(n)
    return v


def torus_maps(Lx, Ly):
    """Site maps of an Lx x Ly periodic square lattice, site = x + Lx y
    (0-based targets, as SpinBasisGeneral's zero-based maps): translations,
    the x reflection, and the spin flip (negative entries, -(target + 1))."""
    def site(x, y):
        return (x % Lx) + Lx * (y % Ly)
    sites = [(x, y) for y in range(Ly) for x in range(Lx)]
    Tx = [site(x + 1, y) for x, y in sites]
    Ty = [site(x, y + 1) for x, y in sites]
    Px = [site(Lx - 1 - x, y) for x, y in sites]
    Z = [-(i + 1) for i in range(Lx * Ly)]
    return Tx, Ty, Px, Z


def torus_heisenberg(Lx, Ly, J=1.0, Jd=0.0):
    """Nearest-neighbour Heisenberg model on the Lx x Ly torus (one-based sites),
    with an optional diagonal coupling Jd (both diagonals)."""
    def site(x, y):
        return (x % Lx) + Lx * (y % Ly) + 1
    bonds = []
    for y in range(Ly):
        for x in range(Lx):
            bonds.append((J, site(x, y), site(x + 1, y)))
            bonds.append((J, site(x, y), site(x, y + 1)))
            if Jd:
                bonds.append((Jd, site(x, y), site(x + 1, y + 1)))
                bonds.append((Jd, site(x, y), site(x + 1, y - 1)))
    return [("+-", [(j / 2, a, b) for j, a, b in bonds]), ("-+", [(j / 2, a, b) for j, a, b in bonds]),
            ("zz", [(j, a, b) for j, a, b in bonds])]


def sublattice(L, J=1.0, J2=0.5, h=0.3):
    """xx on nearest-neighbour bonds, zz on next-nearest bonds, a transverse
    field: commutes with translations, parity and both sublattice flips (zA,
    zB), so it lives in zA / zB sectors (no particle number)."""
    nn = [(i, i % L + 1) for i in range(1, L + 1)]
    nnn = [(i, (i + 1) % L + 1) for i in range(1, L + 1)]
    return [("xx", [(J, a, b) for a, b in nn]), ("zz", [(J2, a, b) for a, b in nnn]),
            ("x", [(h, i) for i in range(1, L + 1)])]
