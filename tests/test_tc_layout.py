"""CPU model of csrc/fused_tc.cu's data path (producer loads, operand images, the GEMMs
the tensor cores compute from them, the epilogue and the adjoint cross term).

For every launch shape it checks that each producer and epilogue access stays inside
the state, each 16-byte chunk of the A image is written once per tile, every amplitude
is read and written exactly once, and that reading the images back with the
SWIZZLE_128B rule and multiplying as the MMA descriptors say reproduces U x (and, for
the adjoint, U^H psi, U^H lam and sum lam conj(psi)^T) against the oracle.
"""
import numpy as np
import pytest

from oracle import statevec as O

A_KB, B_KB = 16384, 8192       # K-block strides of the A (128 rows) and B (64 rows) images
A_IMG, B_IMG = 32768, 16384


def sw128_off(r, chunk, kb_bytes):
    kb, c = chunk >> 3, chunk & 7
    return kb * kb_bytes + (r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4)


def image_read(img, r, k, kb_bytes):
    """Element k of row r of a SWIZZLE_128B K-major bf16 image (one float per 2-byte slot)."""
    return img[(sw128_off(r, k // 8, kb_bytes) + (k % 8) * 2) // 2]


def insert_zero_bits(g, pos):
    for q in sorted(pos):
        g = ((g >> q) << (q + 1)) | (g & ((1 << q) - 1))
    return g


def offsets(tb):
    return [sum(1 << tb[jb] for jb in range(6) if (j >> (5 - jb)) & 1) for j in range(64)]


def build_b(u):
    """k_tc_prep(): row j', K = 64p + j -> part p of U[j'][j]."""
    img = np.full(B_IMG // 2, np.nan)
    for row in range(64):
        for chunk in range(16):
            o = sw128_off(row, chunk, B_KB)
            for e in range(8):
                kk = chunk * 8 + e
                z = u[row, kk & 63]
                img[(o + 2 * e) // 2] = z.imag if kk >> 6 else z.real
    return img


def emulate(states, n, tb, adj, bimg):
    cols = 64 if adj else 128
    offs = offsets(tb)
    out = [s.copy() for s in states]
    cross = np.zeros((128, 128)) if adj else None
    B = np.array([[image_read(bimg, r, k, B_KB) for k in range(128)] for r in range(64)])
    read = [set() for _ in states]
    touched = [set() for _ in states]
    for t in range((1 << (n - 6)) // cols):
        tbase = insert_zero_bits(t * cols, tb)
        aimg = np.full(A_IMG // 2, np.nan)
        written = set()
        for tid in range(256):  # producers: row tid & 127, target patterns 32*gh .. 32*gh+31
            row, gh = tid & 127, tid >> 7
            st = row >> 6 if adj else 0
            ibase = insert_zero_bits(row & 63 if adj else row, tb)
            amps = []
            for e in range(32):
                addr = tbase + ibase + offs[32 * gh + e]
                assert 0 <= addr < (1 << n) and addr not in read[st]
                read[st].add(addr)
                amps.append(states[st][0, addr])
            for h in range(4):
                g = 4 * gh + h
                for part, chunk in ((0, g), (1, 8 + g)):
                    o = sw128_off(row, chunk, A_KB)
                    assert o not in written and o + 16 <= A_IMG
                    written.add(o)
                    for e in range(8):
                        a = amps[8 * h + e]
                        aimg[(o + 2 * e) // 2] = a.imag if part else a.real
        assert not np.isnan(aimg).any()
        A = np.array([[image_read(aimg, i, k, A_KB) for k in range(128)] for i in range(128)])
        d_re = A[:, :64] @ B[:, :64].T - A[:, 64:] @ B[:, 64:].T   # K-block 1 with negate-A
        d_im = A[:, :64] @ B[:, 64:].T + A[:, 64:] @ B[:, :64].T   # B's K-blocks swapped
        if adj:  # MN-major cross term: lam rows 64..127 against psi rows 0..63
            cross += A[64:, :].T @ A[:64, :]
        for sub in range(4):  # epilogue warps: TMEM lanes 32*sub.., one column per lane
            for lane in range(32):
                erow = sub * 32 + lane
                st = erow >> 6 if adj else 0
                ib = insert_zero_bits(erow & 63 if adj else erow, tb)
                for j in range(64):
                    addr = tbase + ib + offs[j]
                    assert addr not in touched[st]
                    touched[st].add(addr)
                    out[st][0, addr] = d_re[erow, j] + 1j * d_im[erow, j]
    for rset, tset in zip(read, touched):
        assert len(rset) == len(tset) == 1 << n
    return out, cross


def _unitary(rng):
    z = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
    return np.linalg.qr(z)[0]


@pytest.mark.parametrize("tb", [[13, 12, 11, 10, 9, 8], [0, 1, 2, 3, 4, 5], [2, 9, 0, 12, 5, 7]])
def test_apply_matches_oracle(tb):
    rng = np.random.default_rng(sum(tb) + 7)
    n = 14
    state = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    u = _unitary(rng)
    out, _ = emulate([state], n, tb, False, build_b(u))
    np.testing.assert_allclose(out[0], O.apply(state, u[None], [n - 1 - b for b in tb], n), atol=1e-10)


@pytest.mark.parametrize("tb", [[13, 12, 11, 10, 9, 8], [2, 9, 0, 12, 5, 7]])
def test_adjoint_matches_oracle(tb):
    rng = np.random.default_rng(sum(tb) + 11)
    n = 14
    wires = [n - 1 - b for b in tb]
    psi = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    lam = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    uh = _unitary(rng).conj().T
    (po, lo), cross = emulate([psi, lam], n, tb, True, build_b(uh))
    np.testing.assert_allclose(po, O.apply(psi, uh[None], wires, n), atol=1e-10)
    np.testing.assert_allclose(lo, O.apply(lam, uh[None], wires, n), atol=1e-10)
    d = cross.reshape(2, 64, 2, 64)  # rows/cols 64p + j (torchquantum_gb300._lib.cross_to_complex)
    m = (d[0, :, 0, :] + d[1, :, 1, :]) + 1j * (d[1, :, 0, :] - d[0, :, 1, :])
    offs = offsets(tb)
    ref = np.zeros((64, 64), dtype=complex)
    for c in range(1 << (n - 6)):
        base = insert_zero_bits(c, tb)
        ref += np.outer(lam[0, [base + o for o in offs]], psi[0, [base + o for o in offs]].conj())
    np.testing.assert_allclose(m, ref, atol=1e-9)
