"""CPU model of csrc/fused_tc.cu's data path: the host's producer mapping and output
orientation (tc_setup), the producers' loads and A-image stores, the U image, the
products the tensor cores compute from the two images in either orientation, both
drains, and the adjoint cross term.

For every launch shape it checks that each load and store stays inside the state and
touches each amplitude exactly once, each 16-byte chunk of the A image is written once
per tile, image stores of a warp fall in distinct 16-byte slots of the SWIZZLE_128B
rows (bank-conflict free), and that reading the images back with the SWIZZLE_128B rule
and multiplying as the MMA descriptors say reproduces U x (and, for the adjoint, U^H psi,
U^H lam and sum lam conj(psi)^T) against the oracle.
"""
import numpy as np
import pytest

from oracle import statevec as O

KB = 16384          # K-block stride of the A and U images (128 rows x 128 B)
IMG = 32768         # one bf16 image (hi or lo)


def sw128_off(r, chunk):
    kb, c = chunk >> 3, chunk & 7
    return kb * KB + (r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4)


def image_read(img, r, k):
    """Element k of row r of a SWIZZLE_128B K-major bf16 image (one float per 2-byte slot)."""
    return img[(sw128_off(r, k // 8) + (k % 8) * 2) // 2]


def insert_zero_bits(g, pos):
    for q in sorted(pos):
        g = ((g >> q) << (q + 1)) | (g & ((1 << q) - 1))
    return g


def pattern_orders(tb):
    """Mirror of pattern_orders(): natural index (bit 5 - jb <-> tb[jb]) of each output-order
    index (bit b = b-th lowest target bit) and each K-order index (b-th highest)."""
    asc = sorted(range(6), key=lambda jb: tb[jb])
    nat = lambda x, order: sum(1 << (5 - order[b]) for b in range(6) if (x >> b) & 1)
    return [nat(x, asc) for x in range(64)], [nat(x, asc[::-1]) for x in range(64)]


def tc_setup(n, tb, adj):
    """Mirror of the host setup: offsets, producer tables and output orientation."""
    tasc = sorted(tb)
    off = [sum(1 << tasc[b] for b in range(6) if (o >> b) & 1) for o in range(64)]
    koff = [sum(1 << tasc[5 - b] for b in range(6) if (jk >> b) & 1) for jk in range(64)]
    ncol = 6 if adj else 7
    colbit = [q for q in range(n) if q not in tb][:ncol]
    col_off = [sum(1 << colbit[c] for c in range(ncol) if ((i & 63 if adj else i) >> c) & 1) for i in range(128)]
    # dims: (addr, off, row, g, lam)
    rest = [(tasc[5 - b], 1 << tasc[5 - b], 0, 1 << (b - 3), 0) for b in range(3, 6)]
    rest += [(colbit[c], 1 << colbit[c], 1 << c, 0, 0) for c in range(ncol)]
    rest.sort(key=lambda d: d[0])
    wdim = rest[7:] + ([(-1, 0, 64, 0, 1)] if adj else [])
    assert len(wdim) == 3

    def table(dims, nbits):
        out = []
        for x in range(1 << nbits):
            sel = [dims[b] for b in range(nbits) if (x >> b) & 1]
            out.append((sum(d[1] for d in sel), sum(d[2] for d in sel), sum(d[3] for d in sel), int(any(d[4] for d in sel))))
        return out

    lanes, warps = table(rest[:5], 5), table(wdim, 3)
    creg = table(rest[5:7], 2)
    reg_off = [koff[r & 7] + creg[r >> 3][0] for r in range(32)]

    def sectors(o):
        return len({x >> 2 for x in o})

    transposed = sectors(off[:16]) < sectors(col_off[:32])
    return dict(off=off, koff=koff, col_off=col_off, lanes=lanes, warps=warps, creg=creg, reg_off=reg_off,
                transposed=transposed, nat_of_k=pattern_orders(tb)[1])


def build_u(u, tb):
    """k_tc_prep(): row 2o [Re U | -Im U], row 2o+1 [Im U | Re U] (K = 64p + jk)."""
    nat_out, nat_k = pattern_orders(tb)
    img = np.full(IMG // 2, np.nan)
    for row in range(128):
        for chunk in range(16):
            o = sw128_off(row, chunk)
            for e in range(8):
                kk = chunk * 8 + e
                z = u[nat_out[row >> 1], nat_k[kk & 63]]
                v = (z.real if kk < 64 else -z.imag) if row % 2 == 0 else (z.imag if kk < 64 else z.real)
                img[(o + 2 * e) // 2] = v
    return img


def emulate(states, n, tb, adj, uimg, transposed=None):
    P = tc_setup(n, tb, adj)
    if transposed is None:
        transposed = P["transposed"]
    cols = 64 if adj else 128
    out = [s.copy() for s in states]
    cross = np.zeros((128, 128)) if adj else None
    Ub = np.array([[image_read(uimg, r, k) for k in range(128)] for r in range(128)])
    read = [set() for _ in states]
    touched = [set() for _ in states]
    for t in range((1 << (n - 6)) // cols):
        tbase = insert_zero_bits(t * cols, tb)
        aimg = np.full(IMG // 2, np.nan)
        written = set()
        for w in range(8):  # producers
            woff, wrow, wg, wlam = P["warps"][w]
            slots = {}
            for l in range(32):
                loff, lrow, lg, _ = P["lanes"][l]
                st = wlam if adj else 0
                vals = []
                for r in range(32):
                    a = tbase + loff + woff + P["reg_off"][r]
                    assert 0 <= a < (1 << n) and a not in read[st]
                    read[st].add(a)
                    vals.append(states[st][0, a])
                for c in range(4):
                    row, g = lrow + wrow + P["creg"][c][1], lg + wg + P["creg"][c][2]
                    assert 0 <= row < 128 and 0 <= g < 8
                    # value e of the chunk is K-order pattern jk = 8g + e of tile row `row`
                    for e in range(8):
                        assert P["col_off"][row] + P["koff"][8 * g + e] == loff + woff + P["reg_off"][8 * c + e]
                    for part, chunk in ((0, g), (1, 8 + g)):
                        o = sw128_off(row, chunk)
                        assert o not in written and o + 16 <= IMG
                        written.add(o)
                        slots.setdefault((c, part), []).append((o % 128) // 16)
                        for e in range(8):
                            v = vals[8 * c + e]
                            aimg[(o + 2 * e) // 2] = v.imag if part else v.real
            for r in range(32):  # one load instruction: 32 lanes x 8 B in at most 8 sectors
                sect = {(tbase + P["lanes"][l][0] + woff + P["reg_off"][r]) >> 2 for l in range(32)}
                assert len(sect) <= 8, (r, len(sect))
            for sl in slots.values():  # one store instruction: 32 lanes, 8 slots x 4 each
                assert sorted(sl) == sorted(list(range(8)) * 4)
        assert not np.isnan(aimg).any()
        A = np.array([[image_read(aimg, i, k) for k in range(128)] for i in range(128)])
        D = A @ Ub.T if not transposed else (Ub @ A.T).T   # D[i][2j' + q] either way
        if adj:  # MN-major cross term: lam rows 64..127 against psi rows 0..63, flushed in natural order
            ck = A[64:, :].T @ A[:64, :]
            nat = [(m & 64) + P["nat_of_k"][m & 63] for m in range(128)]
            cross[np.ix_(nat, nat)] += ck
        for i in range(128):
            st = i >> 6 if adj else 0
            for jp in range(64):
                a = tbase + P["col_off"][i] + P["off"][jp]
                assert a not in touched[st]
                touched[st].add(a)
                out[st][0, a] = D[i, 2 * jp] + 1j * D[i, 2 * jp + 1]
    for rset, tset in zip(read, touched):
        assert len(rset) == len(tset) == 1 << n
    return out, cross


def _unitary(rng):
    z = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
    return np.linalg.qr(z)[0]


LAYOUTS = [[13, 12, 11, 10, 9, 8], [0, 1, 2, 3, 4, 5], [2, 9, 0, 12, 5, 7], [5, 4, 3, 2, 1, 0], [1, 13, 6, 3, 10, 0]]


@pytest.mark.parametrize("tb", LAYOUTS)
def test_apply_matches_oracle(tb):
    rng = np.random.default_rng(sum(tb) + 7)
    n = 14
    state = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    u = _unitary(rng)
    ref = O.apply(state, u[None], [n - 1 - b for b in tb], n)
    for tr in (False, True):
        out, _ = emulate([state], n, tb, False, build_u(u, tb), transposed=tr)
        np.testing.assert_allclose(out[0], ref, atol=1e-10)


@pytest.mark.parametrize("tb", LAYOUTS[:3])
def test_adjoint_matches_oracle(tb):
    rng = np.random.default_rng(sum(tb) + 11)
    n = 14
    wires = [n - 1 - b for b in tb]
    psi = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    lam = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    uh = _unitary(rng).conj().T
    (po, lo), cross = emulate([psi, lam], n, tb, True, build_u(uh, tb))
    np.testing.assert_allclose(po, O.apply(psi, uh[None], wires, n), atol=1e-10)
    np.testing.assert_allclose(lo, O.apply(lam, uh[None], wires, n), atol=1e-10)
    d = cross.reshape(2, 64, 2, 64)  # rows/cols 64p + j (torchquantum_gb300._lib.cross_to_complex)
    m = (d[0, :, 0, :] + d[1, :, 1, :]) + 1j * (d[1, :, 0, :] - d[0, :, 1, :])
    offs = [sum(1 << tb[jb] for jb in range(6) if (j >> (5 - jb)) & 1) for j in range(64)]  # natural order
    ref = np.zeros((64, 64), dtype=complex)
    for c in range(1 << (n - 6)):
        base = insert_zero_bits(c, tb)
        ref += np.outer(lam[0, [base + o for o in offs]], psi[0, [base + o for o in offs]].conj())
    np.testing.assert_allclose(m, ref, atol=1e-9)


def test_orientation_choice():
    """Targets on the lowest address bits store transposed; high targets row-major."""
    assert tc_setup(24, [5, 4, 3, 2, 1, 0], False)["transposed"]
    assert not tc_setup(24, [23, 22, 21, 20, 19, 18], False)["transposed"]
    assert not tc_setup(24, [6, 22, 11, 21, 5, 2], False)["transposed"]
