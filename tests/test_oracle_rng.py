"""Random-number known answers of the oracle (CPU).

Philox4x32-10: the published known-answer vectors of the algorithm (Salmon et
al., SC'11; Random123 kat_vectors).  MT19937: selkov_code/mt95.f90
init_by_scalar (mt95.f90:378-404) is the 2002 init_genrand, checked against
numpy's independent MT19937 (RandomState).  The 1998 sgrnd seeding of
collective_code/mtmod.f90:72-85 and grnd (:88-144) are checked against a
literal Python restatement of the Fortran.
"""
import numpy as np

from oracle import oracle as O


def test_philox_known_answers():
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, out in kat:
        assert [int(v) for v in O.philox(ctr, key)] == out


def test_mt2002_state_matches_numpy():
    for seed in (0, 1, 4357, 5489, 8154543, 2 ** 32 - 1):
        m = O.MT(seed, 2002)
        assert (m.state == np.random.RandomState(seed).get_state()[1]).all()


def test_mt2002_stream_matches_numpy():
    m = O.MT(5489, 2002)
    ours = m.u32(2000)
    theirs = np.random.RandomState(5489).randint(0, 2 ** 32, size=2000, dtype=np.uint64).astype(np.uint32)
    assert (ours == theirs).all()
    assert int(ours[0]) == 3499211612      # first output of MT19937 seeded 5489


def test_mt95_real1_mapping():
    # genrand_real1 = signed32 * 1/(2^32-1) + 2^31/(2^32-1)  (mt95.f90:828-841)
    a = O.MT(8154543, 2002)
    b = O.MT(8154543, 2002)
    words = b.u32(50)
    for w in words:
        s = int(w) - (1 << 32) if w >= 2 ** 31 else int(w)
        ref = s * (1.0 / (4294967296.0 - 1.0)) + 2147483648.0 / (4294967296.0 - 1.0)
        assert a.real1() == ref


def _mtmod_restated(seed, n):
    """Literal restatement of mtmod.f90 sgrnd + grnd with 32-bit wraparound."""
    N, M = 624, 397
    mask = 0xFFFFFFFF
    mt = [seed & mask]
    for i in range(1, N):
        mt.append((69069 * mt[i - 1]) & mask)
    mti = N
    out = []
    for _ in range(n):
        if mti >= N:
            for kk in range(N):
                y = (mt[kk] & 0x80000000) | (mt[(kk + 1) % N] & 0x7FFFFFFF)
                mt[kk] = mt[(kk + M) % N] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            mti = 0
        y = mt[mti]
        mti += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        out.append(y / (4294967296.0 - 1.0))
    return out


def test_mt1998_grnd_restated():
    for seed in (4357, 345342763, 123456789):
        m = O.MT(seed, 1998)
        ref = _mtmod_restated(seed, 1500)
        got = [m.grnd() for _ in range(1500)]
        assert got == ref


def test_contract_stream_properties():
    u = np.array([O.contract_u01(1, 2, i, 0, 50, i & 1) for i in range(20000)])
    assert (u >= 0).all() and (u < 1).all()
    assert abs(u.mean() - 0.5) < 0.01
    assert abs(u.var() - 1 / 12) < 0.002
