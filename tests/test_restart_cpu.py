"""CPU checks of the restart particle section and the particle checksum.

The reference's CRC32 class (src/general/specfunc.h:438-505) cannot be built
here (specfunc.h needs MPI), so the oracle's restatement is pinned by
 - the published check value of the MSB-first 0x04C11DB7 CRC with initial
   value 0 and no reflection: CRC-32/POSIX gives 0x765E7680 for "123456789"
   after its final xor with 0xFFFFFFFF, so the low half here is 0x89A1897F;
 - a second, independent restatement of the 64-bit accumulator recurrence
   (the class keeps the bits shifted above bit 31 in an unsigned long).
The device combines per-record CRCs with the append operator and replays the
last record on the host; that combination is emulated here with numpy and
checked against the oracle's sequential walk.
"""
import numpy as np

from amps_gb300._capi import RecordLayout
from tests import oracle_lib as O

MASK64 = (1 << 64) - 1


def _table64():
    t = []
    for i in range(256):
        a = i << 24
        for _ in range(8):
            a = ((a << 1) ^ 0x04C11DB7) if (a & 0x80000000) else (a << 1)
        t.append(a & MASK64)
    return t


T64 = _table64()


def crc64_py(acc, data):
    for b in bytes(data):
        acc = ((acc << 8) ^ T64[((acc >> 24) ^ b) & 0xFF]) & MASK64
    return acc


def test_crc_low_half_matches_published_check_value():
    assert O.crc32_add(0, b"123456789") & 0xFFFFFFFF == 0x89A1897F
    assert crc64_py(0, b"123456789") & 0xFFFFFFFF == 0x89A1897F


def test_crc_accumulator_matches_independent_restatement():
    rng = np.random.default_rng(1)
    for n in (1, 3, 4, 5, 65, 80, 1000):
        data = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        acc0 = int(rng.integers(0, 2 ** 32))
        assert O.crc32_add(acc0, data) == crc64_py(acc0, data)
    # the high half is not zero: it keeps the shifted-out bits
    assert O.crc32_add(0, b"123456789") >> 32 != 0
    # chaining two adds is one add over the concatenation
    a, b = b"restart-", b"particles"
    assert O.crc32_add(O.crc32_add(0, a), b) == O.crc32_add(0, a + b)


def _records(n, layout, seed):
    rng = np.random.default_rng(seed)
    nb = 3
    block = rng.integers(0, nb, n).astype(np.int32)
    cell = rng.integers(0, 512, n).astype(np.int32)
    x = rng.uniform(-5, 5, (n, 3))
    v = rng.standard_normal((n, 3))
    spec = rng.integers(0, 2, n).astype(np.uint8)
    wc = rng.uniform(0.5, 2, n) if layout.off_weight >= 0 else None
    return nb, x, v, spec, block, cell, wc


def _rec_bytes(layout, x, v, s, w):
    r = bytearray(layout.record_length)
    r[layout.off_velocity:layout.off_velocity + 24] = np.asarray(v, np.float64).tobytes()
    r[layout.off_position:layout.off_position + 24] = np.asarray(x, np.float64).tobytes()
    r[layout.off_species] = int(s)
    if layout.off_weight >= 0:
        r[layout.off_weight:layout.off_weight + 8] = np.float64(w).tobytes()
    return bytes(r)


def _gf2_apply(cols, x):
    y = 0
    for b in range(32):
        if (x >> b) & 1:
            y ^= cols[b]
    return y


def _gf2_mul(a, b):
    return [_gf2_apply(a, c) for c in b]


def _gf2_pow(m, e):
    r = [1 << k for k in range(32)]
    while e:
        if e & 1:
            r = _gf2_mul(m, r)
        m = _gf2_mul(m, m)
        e >>= 1
    return r


def test_device_combination_equals_sequential_walk():
    """per-record CRC from zero, append operator Z^len, chunks of 256 records,
    the last record replayed in the 64-bit accumulator: the device's algorithm"""
    for layout in (RecordLayout.basic(False), RecordLayout.basic(True)):
        n = 1500
        nb, x, v, spec, block, cell, wc = _records(n, layout, 7)
        # list order = input order within each (block, cell); checksum order:
        # blocks, cells i-major, list order
        i, j, k = cell % 8, (cell // 8) % 8, cell // 64
        order = np.lexsort((np.arange(n), i * 64 + j * 8 + k, block))
        recs = [_rec_bytes(layout, x[p], v[p], spec[p], 1.0 if wc is None else wc[p]) for p in order]
        lo = [t & 0xFFFFFFFF for t in T64]
        zero = [((1 << kk) << 8 & 0xFFFFFFFF) ^ lo[(1 << kk) >> 24] for kk in range(32)]
        M = _gf2_pow(zero, layout.record_length)
        crc = [crc64_py(0, r) & 0xFFFFFFFF for r in recs]
        chunk = 256
        MC = _gf2_pow(M, chunk)
        acc = 0
        body = crc[:-1]
        for c0 in range(0, len(body), chunk):
            part = body[c0:c0 + chunk]
            s = 0
            for c in part:
                s = _gf2_apply(M, s) ^ c
            acc = _gf2_apply(MC if len(part) == chunk else _gf2_pow(M, len(part)), acc) ^ s
        total = crc64_py(acc, recs[-1])
        want = O.particle_checksum(layout, nb, x, v, spec, block, cell, wc)
        assert total == want
        assert want == crc64_py(0, b"".join(recs))


def test_section_layout_of_the_oracle_pack():
    layout = RecordLayout.basic(True)
    n = 700
    nb, x, v, spec, block, cell, wc = _records(n, layout, 9)
    block[block == 1] = 2                     # block 1 holds no particles: not written
    order = np.array([2, 0, 1], np.int32)
    ids = np.array([[7, 0, 0, 0], [8, 0, 0, 0], [9, 0, 0, 0]], np.uint8)
    w = [0.25, 4.0]
    sec = O.restart_pack(layout, nb, x, v, spec, block, cell, w, wc, order, ids).tobytes()
    assert sec[:43] == b"PARTICLE-RESTART-FILE--END-USER-ADDITIONAL\x00"
    assert np.frombuffer(sec[43:51], np.int64)[0] == 80
    assert np.frombuffer(sec[51:67], np.float64).tolist() == w
    pos = 67
    seen = []
    for b in order:
        sel = np.flatnonzero(block == b)
        if sel.size == 0:
            continue
        assert sec[pos:pos + 4] == ids[b].tobytes()
        tot = int(np.frombuffer(sec[pos + 4:pos + 8], np.int32)[0])
        table = np.frombuffer(sec[pos + 8:pos + 8 + 2048], np.int32).reshape(8, 8, 8)
        assert tot == sel.size == table.sum()
        pos += 8 + 2048
        for ii in range(8):
            for jj in range(8):
                for kk in range(8):
                    lst = sel[cell[sel] == ii + 8 * (jj + 8 * kk)]   # list order
                    assert table[ii, jj, kk] == lst.size
                    for p in lst[::-1]:                               # tail first
                        assert sec[pos:pos + 80] == _rec_bytes(layout, x[p], v[p], spec[p], wc[p])
                        pos += 80
        seen.append(b)
    assert pos == len(sec) and seen == [2, 0]
