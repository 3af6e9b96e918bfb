"""CPU model of csrc/fused_tc.cu's data layout: tile load mapping, SWIZZLE_128B K-major
operand images, the GEMM the tensor cores compute from those images, and the epilogue.

Checks that (a) every shared-memory write stays inside its 32 KB image and each
16-byte chunk is written once, (b) every global access stays inside its row and each
amplitude of a tile is loaded and stored exactly once, (c) reading the images back
with the swizzle rule and multiplying reproduces U x for every column (exact in
float64), against the oracle's gate application.
"""
import numpy as np
import pytest

from oracle import statevec as O

IMG = 32768
KB = 16384


def sw128_off(r, chunk):
    kb, c = chunk >> 3, chunk & 7
    return kb * KB + (r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4)


def insert_zero_bits(g, pos):
    for q in sorted(pos):
        g = ((g >> q) << (q + 1)) | (g & ((1 << q) - 1))
    return g


def offsets(tb):
    return [sum(1 << tb[jb] for jb in range(6) if (j >> (5 - jb)) & 1) for j in range(64)]


def image_read(img, r, k):
    """Element k of row r from a SWIZZLE_128B K-major image stored as 2-element float slots."""
    return img[(sw128_off(r, k // 8) + (k % 8) * 2) // 2]


def build_a(state_row, c0, tb, offs):
    """produce(): 2048 (column, quad) pairs -> float image (one float per bf16 slot)."""
    img = np.full(IMG // 2, np.nan)
    seen_chunks = set()
    loaded = []
    for e in range(128 * 16):
        i, q = e & 127, e >> 7
        base = insert_zero_bits(c0 + i, tb)
        amps = [state_row[base + offs[4 * q + r]] for r in range(4)]
        loaded += [base + offs[4 * q + r] for r in range(4)]
        o = sw128_off(i, q)
        assert 0 <= o and o + 16 <= IMG and o % 16 == 0
        assert o not in seen_chunks
        seen_chunks.add(o)
        for r, a in enumerate(amps):
            img[(o + 4 * r) // 2] = a.real
            img[(o + 4 * r + 2) // 2] = a.imag
    return img, loaded


def build_b(u):
    """k_tc_prep(): real embedding rows n=2j'+p', K=2j+p."""
    img = np.full(IMG // 2, np.nan)
    for n in range(128):
        jo, po = n >> 1, n & 1
        for chunk in range(16):
            o = sw128_off(n, chunk)
            for e in range(8):
                kk = chunk * 8 + e
                j, pi = kk >> 1, kk & 1
                z = u[jo, j]
                v = (z.real if pi == 0 else -z.imag) if po == 0 else (z.imag if pi == 0 else z.real)
                img[(o + 2 * e) // 2] = v
    return img


@pytest.mark.parametrize("tb_choice", [[13, 12, 11, 10, 9, 8], [0, 1, 2, 3, 4, 5], [2, 9, 0, 12, 5, 7]])
def test_tc_tile_roundtrip_matches_oracle(tb_choice):
    rng = np.random.default_rng(sum(tb_choice))
    n = 14
    tb = tb_choice  # bit of matrix-index bit j (j=0 is the MSB)
    wires = [n - 1 - b for b in tb]
    state = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    state /= np.linalg.norm(state)
    z = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
    u, _ = np.linalg.qr(z)
    offs = offsets(tb)
    bimg = build_b(u)
    assert not np.isnan(bimg).any()
    tiles_per_row = (1 << (n - 6)) // 128
    out = state.copy()
    touched = []
    for t in range(tiles_per_row):
        c0 = t * 128
        aimg, loaded = build_a(state[0], c0, tb, offs)
        assert not np.isnan(aimg).any()
        assert all(0 <= a < (1 << n) for a in loaded)
        # D[i][n] = sum_K A[i][K] B[n][K], reading both images through the swizzle rule
        A = np.array([[image_read(aimg, i, k) for k in range(128)] for i in range(128)])
        B = np.array([[image_read(bimg, nn, k) for k in range(128)] for nn in range(128)])
        D = A @ B.T
        # epilogue: warp w -> lanes (rows) 32*(w%4)+lane, columns half*64 + [0,64)
        for w in range(8):
            sub, half = w & 3, w >> 2
            for lane in range(32):
                i = sub * 32 + lane
                base = insert_zero_bits(c0 + i, tb)
                for col in range(half * 64, half * 64 + 64, 2):
                    j = col >> 1
                    out[0, base + offs[j]] = D[i, col] + 1j * D[i, col + 1]
                    touched.append(base + offs[j])
        assert sorted(loaded) == sorted(set(loaded))
    assert sorted(touched) == list(range(1 << n))
    ref = O.apply(state, u[None], wires, n)
    np.testing.assert_allclose(out, ref, atol=1e-12)


# ---------------------------------------------------------------- v2 (cp.async staging)
def stage_chunk(c):
    return c ^ ((c >> 5) & 31)


def tc_setup(n, tb, adj):
    used = sum(1 << b for b in tb)
    ncol = 6 if adj else 7
    colbits = [q for q in range(n) if not (used >> q) & 1][:ncol]
    sbits = sorted(set(tb) | set(colbits))
    col_pos = [sbits.index(b) for b in colbits]
    tgt_pos = [sbits.index(b) for b in tb]
    return sbits, col_pos, tgt_pos


def scatter(u, sbits):
    return sum(1 << sbits[b] for b in range(len(sbits)) if (u >> b) & 1)


def emulate_v2(states, n, tb, adj, bimg):
    """Run the v2 data path for every tile; returns (outputs per state, cross term or None)."""
    sbits, col_pos, tgt_pos = tc_setup(n, tb, adj)
    assert sbits[0] == 0  # 16-byte chunks hold address-adjacent amplitude pairs
    cols = 64 if adj else 128
    nbits = 12 if adj else 13
    chunks = 1 << (nbits - 1)
    offs = offsets(tb)
    uj = [sum(1 << tgt_pos[jb] for jb in range(6) if (j >> (5 - jb)) & 1) for j in range(64)]
    schunk = [scatter(512 * s, sbits) for s in range(16)]
    out = [s.copy() for s in states]
    tiles = (1 << (n - 6)) // cols
    cross = np.zeros((128, 128)) if adj else None
    B = np.array([[image_read(bimg, nn, k) for k in range(128)] for nn in range(128)])
    for t in range(tiles):
        c0 = t * cols
        tbase = insert_zero_bits(c0, tb)
        stage = [np.full(chunks * 2, np.nan, dtype=np.complex128) for _ in range(2 if adj else 1)]
        for tid in range(256):
            a_tid = scatter(2 * tid, sbits)
            for s in range(16):
                st, sl = (s >> 3, s & 7) if adj else (0, s)
                c = tid + 256 * sl
                g = tbase + a_tid + schunk[sl]
                assert g == tbase + scatter(2 * c, sbits) and g % 2 == 0 and g + 1 < (1 << n)
                ph = stage_chunk(c)
                assert 0 <= ph < chunks
                assert np.isnan(stage[st][2 * ph])
                stage[st][2 * ph] = states[st][0, g]
                stage[st][2 * ph + 1] = states[st][0, g + 1]
        aimg = np.full(IMG // 2, np.nan)
        for tid in range(256):
            crow = tid & 127
            ccol = crow & 63 if adj else crow
            st = crow >> 6 if adj else 0
            ucol = sum(1 << col_pos[b] for b in range(6 if adj else 7) if (ccol >> b) & 1)
            for s in range(8):
                q = (tid >> 7) + 2 * s
                o = sw128_off(crow, q)
                for r in range(4):
                    u = ucol | uj[4 * q + r]
                    a = stage[st][stage_chunk(u >> 1) * 2 + (u & 1)]
                    assert not np.isnan(a)
                    aimg[(o + 4 * r) // 2] = a.real
                    aimg[(o + 4 * r + 2) // 2] = a.imag
        assert not np.isnan(aimg).any()
        A = np.array([[image_read(aimg, i, k) for k in range(128)] for i in range(128)])
        D = A @ B.T
        if adj:  # cross term: lam rows 64..127 against psi rows 0..63
            cross += np.array([[sum(A[64 + i, m] * A[i, nn] for i in range(64)) for nn in range(128)]
                               for m in range(128)])
        for tid in range(256):
            warp, lane = tid >> 5, tid & 31
            sub, half = warp & 3, warp >> 2
            erow = sub * 32 + lane
            st = erow >> 6 if adj else 0
            ib = insert_zero_bits(erow & 63 if adj else erow, tb)
            for col in range(half * 64, half * 64 + 64, 2):
                j = col >> 1
                out[st][0, tbase + ib + offs[j]] = D[erow, col] + 1j * D[erow, col + 1]
    return out, cross


@pytest.mark.parametrize("tb", [[13, 12, 11, 10, 9, 8], [0, 1, 2, 3, 4, 5], [2, 9, 0, 12, 5, 7]])
def test_v2_apply_matches_oracle(tb):
    rng = np.random.default_rng(sum(tb) + 7)
    n = 14
    wires = [n - 1 - b for b in tb]
    state = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    z = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
    u, _ = np.linalg.qr(z)
    out, _ = emulate_v2([state], n, tb, False, build_b(u))
    np.testing.assert_allclose(out[0], O.apply(state, u[None], wires, n), atol=1e-10)


@pytest.mark.parametrize("tb", [[13, 12, 11, 10, 9, 8], [2, 9, 0, 12, 5, 7]])
def test_v2_adjoint_matches_oracle(tb):
    rng = np.random.default_rng(sum(tb) + 11)
    n = 14
    wires = [n - 1 - b for b in tb]
    psi = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    lam = rng.normal(size=(1, 1 << n)) + 1j * rng.normal(size=(1, 1 << n))
    z = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
    u, _ = np.linalg.qr(z)
    uh = u.conj().T
    (po, lo), cross = emulate_v2([psi, lam], n, tb, True, build_b(uh))
    np.testing.assert_allclose(po, O.apply(psi, uh[None], wires, n), atol=1e-10)
    np.testing.assert_allclose(lo, O.apply(lam, uh[None], wires, n), atol=1e-10)
    # M[j][j'] = sum_cols lam[j] conj(psi[j'])
    d = cross.reshape(64, 2, 64, 2)
    m = (d[:, 0, :, 0] + d[:, 1, :, 1]) + 1j * (d[:, 1, :, 0] - d[:, 0, :, 1])
    offs = offsets(tb)
    ref = np.zeros((64, 64), dtype=complex)
    for c in range(1 << (n - 6)):
        base = insert_zero_bits(c, tb)
        lv = lam[0, [base + offs[j] for j in range(64)]]
        pv = psi[0, [base + offs[j] for j in range(64)]]
        ref += np.outer(lv, pv.conj())
    np.testing.assert_allclose(m, ref, atol=1e-9)
