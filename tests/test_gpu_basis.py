"""Device basis vs the oracle: enumeration, representatives, normalisations,
amplitudes and indices are bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SECTORS = [
    (4, 2, dict()),
    (10, 5, dict()),
    (10, None, dict()),
    (8, 4, dict(kblock=0)),
    (8, 4, dict(kblock=1)),
    (8, 4, dict(kblock=4, pblock=1)),
    (10, 5, dict(kblock=0, pblock=1)),
    (10, 5, dict(kblock=0, pblock=-1, zblock=1)),
    (12, 6, dict(kblock=0, pblock=1)),
    (12, 6, dict(kblock=0, pblock=1, zblock=1)),
    (12, 6, dict(kblock=0, pblock=-1, zblock=-1)),
    (12, 6, dict(kblock=6, pblock=1, zblock=1)),
    (12, 6, dict(kblock=3)),
    (12, 6, dict(kblock=2, zblock=-1)),
    (12, 6, dict(pblock=1, zblock=1)),
    (12, 6, dict(pzblock=1)),
    (12, None, dict(kblock=0, pblock=1)),
    (12, None, dict(kblock=0, zAblock=1, a=2)),
    (11, None, dict(kblock=0, pblock=-1, zblock=1)),
    (14, 7, dict(kblock=0, pblock=1, zblock=1)),
    (14, 7, dict(kblock=5, zblock=1)),
    (16, 8, dict(kblock=0, pblock=1, zblock=1)),
    (9, 4, dict(kblock=3, a=3)),
    # sublattice flips (src/basis.jl:740-741): zB alone, with zA, with T(a=2)
    (12, None, dict(zBblock=1)),
    (12, None, dict(zBblock=-1)),
    (12, None, dict(zAblock=1, zBblock=-1)),
    (12, None, dict(kblock=0, zBblock=-1, a=2)),
    (12, None, dict(kblock=0, zAblock=-1, zBblock=1, a=2)),
    (14, None, dict(kblock=3, zAblock=1, zBblock=1, a=2)),
]


@pytest.mark.parametrize("L,nup,kw", SECTORS)
def test_basis_matches_oracle(qs, ora, L, nup, kw):
    ref = ora.RefBasis(L, nup=nup, pauli=False, **kw)
    b = qs.SpinBasis1D(L, nup=nup, pauli=False, **kw)
    assert b.Ns == ref.Ns
    # representatives: bit-exact, in column order
    assert np.array_equal(b.states, ref.states)
    # orbit minima ascending == the representative-space restatement
    rep = ora.RepBasis(L, nup=nup, pauli=False, **kw)
    assert np.array_equal(b.orbit_minima(), rep.states)
    # state_index on every representative; non-representatives are rejected
    idx = b.index_array(ref.states)
    assert np.array_equal(idx, np.arange(b.Ns))
    # representative / normalization / get_amp for every parent state: bit-exact
    reps, norms, amps, status = b.representative_array(ref.parent_states)
    for i, s in enumerate(ref.parent_states):
        try:
            r, nrm, amp = ref.representative(int(s))
        except ora.OracleError:
            assert status[i] == 2
            continue
        assert status[i] == 0
        assert int(reps[i]) == r
        assert norms[i] == nrm, (s, norms[i], nrm)
        assert amps[i] == amp, (s, amps[i], amp)


def test_state_queries(qs):
    b = qs.SpinBasis1D(4, nup=2, pauli=False)
    assert sorted(int(s) for s in b.states) == [3, 5, 6, 9, 10, 12]
    for s in b.states:
        assert qs.state_at(b, qs.state_index(b, int(s))) == s
        assert qs.state_to_int(b, qs.int_to_state(b, int(s))) == s
    assert qs.int_to_state(b, 5, bracket_notation=False) == "0101"
    with pytest.raises(qs.ArgumentError):
        qs.state_index(b, 0)


def test_large_sector_dimensions(qs):
    # exact Burnside counts of the workload sectors
    assert qs.SpinBasis1D(16, nup=8, pauli=False).Ns == 12870
    b = qs.SpinBasis1D(26, nup=13, pauli=False, kblock=1)
    assert b.Ns == 400023
    b = qs.SpinBasis1D(26, nup=13, pauli=False, kblock=0, pblock=1)
    assert b.Ns == 200474
