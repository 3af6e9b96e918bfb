"""CPU model of the kernels' thread -> amplitude index mapping (csrc/apply.cu,
csrc/measure.cu).  For every launch shape the host code picks, checks that each
access is inside the row, that float4 accesses are 16-byte aligned, and that the
gate's amplitude groups are covered exactly once; for the coset passes of the Pauli
strings, that the staged cosets partition each row and that the stage-coordinate
partner and sign rules reproduce the in-row ones."""
import itertools

import numpy as np
import pytest

from oracle import statevec as O


def insert_zero_bits(g, pos):
    for q in sorted(pos):
        lo = g & ((1 << q) - 1)
        g = ((g >> q) << (q + 1)) | lo
    return g


def dense_accesses(n, tbits, cbits):
    """Addresses touched by k_dense<D, MODE> for targets tbits (matrix MSB first), controls cbits."""
    kt = len(tbits)
    D = 1 << kt
    touched = set(tbits) | set(cbits)
    groups = 1 << (n - len(touched))
    setmask = sum(1 << c for c in cbits)
    off = []
    for r in range(D):
        o = 0
        for j in range(kt):
            if (r >> (kt - 1 - j)) & 1:
                o |= 1 << tbits[j]
        off.append(o)
    bit0_ctrl = 0 in cbits
    bit0_tgt = 0 in tbits
    mode = "scl" if bit0_ctrl else ("low" if bit0_tgt else "vec")
    pair = [-1] * D
    if mode == "low":
        for r in range(D):
            if off[r] & 1 == 0:
                for r2 in range(D):
                    if off[r2] == off[r] | 1:
                        pair[r] = r2
    acc = []
    pairs = (groups + 1) >> 1
    for t in range(pairs):
        g0 = 2 * t
        two = g0 + 1 < groups
        if mode == "vec":
            base = insert_zero_bits(g0, touched) | setmask
            for r in range(D):
                a = base + off[r]
                assert a % 2 == 0, "float4 access must be 16-byte aligned"
                acc += [a, a + 1]
        else:
            for j in range(2):
                if j == 1 and not two:
                    break
                base = insert_zero_bits(g0 + j, touched) | setmask
                for r in range(D):
                    if mode == "low":
                        if pair[r] >= 0:
                            a = base + off[r]
                            assert a % 2 == 0
                            acc += [a, a + 1]
                    else:
                        acc.append(base + off[r])
    return acc, setmask, touched


def expected_group_amps(n, tbits, cbits):
    want = []
    for i in range(1 << n):
        if all((i >> c) & 1 for c in cbits):
            want.append(i)
    return want


@pytest.mark.parametrize("n", [1, 2, 3, 4, 6])
def test_dense_1_and_2_target_cover_exactly_once(n):
    bits = list(range(n))
    for kt in (1, 2):
        for tb in itertools.permutations(bits, kt):
            rest = [b for b in bits if b not in tb]
            for nc in range(0, min(2, len(rest)) + 1):
                for cb in itertools.combinations(rest, nc):
                    acc, _, _ = dense_accesses(n, list(tb), list(cb))
                    assert all(0 <= a < (1 << n) for a in acc)
                    assert sorted(acc) == expected_group_amps(n, tb, cb), (n, tb, cb)


def mcx_accesses(n, cbits, tbit, ctrl_val):
    touched = set(cbits) | {tbit}
    groups = 1 << (n - len(touched))
    setmask = sum(1 << c for c in cbits) if ctrl_val else 0
    bit0_ctrl, bit0_tgt = 0 in cbits, tbit == 0
    mode = "scl" if bit0_ctrl else ("low" if bit0_tgt else "vec")
    work = groups // 2 if mode == "vec" else groups
    acc = []
    for t in range(work):
        if mode == "vec":
            i0 = insert_zero_bits(2 * t, touched) | setmask
            assert i0 % 2 == 0 and (i0 | (1 << tbit)) % 2 == 0
            acc += [i0, i0 + 1, i0 | (1 << tbit), (i0 | (1 << tbit)) + 1]
        elif mode == "low":
            i0 = insert_zero_bits(t, touched) | setmask
            assert i0 % 2 == 0
            acc += [i0, i0 + 1]
        else:
            i0 = insert_zero_bits(t, touched) | setmask
            acc += [i0, i0 | (1 << tbit)]
    return acc


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_mcx_covers_controlled_pairs(n):
    bits = list(range(n))
    for tb in bits:
        rest = [b for b in bits if b != tb]
        for nc in range(0, min(3, len(rest)) + 1):
            for cb in itertools.combinations(rest, nc):
                for cv in (0, 1):
                    acc = mcx_accesses(n, list(cb), tb, cv)
                    want = [i for i in range(1 << n) if all(((i >> c) & 1) == cv for c in cb)]
                    assert sorted(acc) == want, (n, tb, cb, cv)


@pytest.mark.parametrize("n", [2, 3, 5])
def test_swap_and_phase_cover(n):
    bits = list(range(n))
    for b0, b1 in itertools.permutations(bits, 2):
        touched = {b0, b1}
        groups = 1 << (n - 2)
        vec = 0 not in touched
        acc = []
        for t in range(groups // 2 if vec else groups):
            if vec:
                base = insert_zero_bits(2 * t, touched)
                for a in (base | (1 << b1), base | (1 << b0)):
                    assert a % 2 == 0
                    acc += [a, a + 1]
            else:
                base = insert_zero_bits(t, touched)
                acc += [base | (1 << b1), base | (1 << b0)]
        want = [i for i in range(1 << n) if ((i >> b0) & 1) != ((i >> b1) & 1)]
        assert sorted(acc) == want
    for k in range(0, n + 1):
        for wb in itertools.combinations(bits, k):
            touched = set(wb)
            groups = 1 << (n - k)
            vec = 0 not in touched
            mask = sum(1 << b for b in wb)
            acc = []
            for t in range(groups // 2 if vec else groups):
                i0 = insert_zero_bits(2 * t if vec else t, touched) | mask
                acc += [i0, i0 + 1] if vec else [i0]
            assert sorted(acc) == [i for i in range(1 << n) if i & mask == mask]


@pytest.mark.parametrize("n", [1, 2, 3, 4, 6])
def test_expval_pair_iteration_covers_each_pair_once(n):
    for x in range(1, 1 << n):
        h = x.bit_length() - 1
        seen = []
        if x == 1:
            for t in range((1 << n) >> 1):
                i = 2 * t
                seen += [(i, i + 1)]
        else:
            lomask = (1 << h) - 1
            for t in range((1 << n) >> 2):
                g = 2 * t
                i = ((g >> h) << (h + 1)) | (g & lomask)
                ip = i ^ x
                assert i % 2 == 0 and 0 <= (ip & ~1) < (1 << n)
                seen += [(i, ip), (i + 1, ip ^ 1)]
        want = sorted((i, i ^ x) for i in range(1 << n) if not (i >> h) & 1)
        assert sorted(seen) == want, x


def test_dense_k_groups_per_block_fit_shared_memory():
    for k in range(1, 13):
        D = 1 << k
        gpb = 1 if D >= 256 else 256 // D
        assert gpb * D <= 16 * 256
        assert gpb * D * 8 <= 200 * 1024


def _popc(v):
    return bin(int(v)).count("1")


def _pauli_apply(psi, x, z):
    """(P psi)[i] = i^ny (-1)^popcount((i ^ x) & z) psi[i ^ x], ny = popcount(x & z) mod 4."""
    ph = [1, 1j, -1, -1j][_popc(x & z) & 3]
    return [ph * (-1) ** _popc((i ^ x) & z) * psi[i ^ x] for i in range(len(psi))]


def test_expval_pass_sign_algebra():
    """The per-pass formulas of k_expval_diag / k_expval_pair (one popcount per string for
    two pairs, sign of the partner from ny, of the odd index from z & 1) against
    <psi|P|psi> computed directly."""
    import numpy as np

    rng = np.random.default_rng(0)
    n = 1 << 6
    for trial in range(200):
        psi = rng.normal(size=n) + 1j * rng.normal(size=n)
        x = 0 if trial % 5 == 0 else 1 if trial % 7 == 0 else int(rng.integers(0, n))
        z = int(rng.integers(0, n))
        ny = _popc(x & z) & 3
        f, z0 = (1 if ny < 2 else -1), (-1 if z & 1 else 1)
        acc = 0.0
        if x == 0:
            for i in range(0, n, 2):
                acc += (-1) ** _popc(i & z) * (abs(psi[i]) ** 2 + z0 * abs(psi[i + 1]) ** 2)
        elif x == 1:
            for i in range(0, n, 2):
                u = np.conj(psi[i]) * psi[i + 1]
                acc += 2 * f * (-1) ** _popc(i & z) * (u.imag if ny & 1 else u.real)
        else:
            hb = x.bit_length() - 1
            for t in range(n // 4):
                g = 2 * t
                i = ((g >> hb) << (hb + 1)) | (g & ((1 << hb) - 1))
                u0 = np.conj(psi[i]) * psi[i ^ x]
                u1 = np.conj(psi[i + 1]) * psi[(i + 1) ^ x]
                c = (u0.imag + z0 * u1.imag) if ny & 1 else (u0.real + z0 * u1.real)
                acc += 2 * f * (-1) ** _popc(i & z) * c
        want = np.vdot(psi, _pauli_apply(psi, x, z)).real
        assert abs(acc - want) < 1e-10, (x, z)


def test_apply_sum_sign_algebra():
    """The backward seed's per-string step (k_coset<true>: sign from one popcount plus
    ny >> 1, quarter turn for odd ny, the odd index of a pair flipped by z & 1) against
    sum_s c_s P_s psi, in in-row coordinates."""
    import numpy as np

    rng = np.random.default_rng(1)
    n = 1 << 6
    for _ in range(40):
        psi = rng.normal(size=n) + 1j * rng.normal(size=n)
        k = int(rng.integers(1, 9))
        xs, zs, cs = rng.integers(0, n, k), rng.integers(0, n, k), rng.normal(size=k)
        got = np.zeros(n, complex)
        for t in range(n // 2):
            i = 2 * t
            for x, z, c in zip(xs, zs, cs):
                x, z = int(x), int(z)
                ny = _popc(x & z) & 3
                c0 = c * (-1) ** (_popc((i ^ x) & z) + (ny >> 1))
                c1 = -c0 if z & 1 else c0
                rot = 1j if ny & 1 else 1
                got[i] += c0 * rot * psi[i ^ x]
                got[i + 1] += c1 * rot * psi[(i + 1) ^ x]
        want = sum(c * np.array(_pauli_apply(psi, int(x), int(z))) for x, z, c in zip(xs, zs, cs))
        assert np.abs(got - want).max() < 1e-10


# ------------------------------------------------------------------ coset passes (measure.cu)
def _reduced_basis(vectors):
    """Reduced echelon basis (ascending pivots), as gf2_reduced_basis in measure.cu."""
    basis = []  # [pivot, vector]
    for v in vectors:
        for piv, b in basis:
            if (v >> piv) & 1:
                v ^= b
        if v == 0:
            continue
        q = v.bit_length() - 1
        basis = [[piv, b ^ v if (b >> q) & 1 else b] for piv, b in basis]
        basis.append([q, v])
    basis.sort()
    return [b for _, b in basis], [piv for piv, _ in basis]


def _coset_model(n, xs, zs, group, c):
    """For one coset pass: list over (coset t) of (global in-row index of each stage
    coordinate u, per-string partner stage coordinate, per-string sign bit of u), built
    from the same algebra as k_coset / coset_params."""
    basis, piv = _reduced_basis([xs[j] >> c for j in group])
    r = len(basis)
    lmask = (1 << c) - 1
    consts = []
    for j in group:
        xh, zh = xs[j] >> c, zs[j] >> c
        a = sum(1 << k for k in range(r) if (xh >> piv[k]) & 1)
        beta = sum(1 << k for k in range(r) if bin(basis[k] & zh).count("1") & 1)
        consts.append(((a << c) | (xs[j] & lmask), (beta << c) | (zs[j] & lmask), zh))
    out = []
    for t in range(1 << (n - c - r)):
        rep = t
        for q in piv:
            rep = ((rep >> q) << (q + 1)) | (rep & ((1 << q) - 1))
        gidx = []
        for u in range(1 << (c + r)):
            a, l = u >> c, u & lmask
            h = rep
            for k in range(r):
                if (a >> k) & 1:
                    h ^= basis[k]
            gidx.append((h << c) | l)
        rho = [bin(rep & zh).count("1") & 1 for _, _, zh in consts]
        out.append((gidx, consts, rho))
    return out, r


@pytest.mark.parametrize("n,m,seed", [(5, 4, 0), (9, 6, 1), (14, 8, 2), (15, 12, 3), (16, 20, 4)])
def test_coset_partition_partners_and_signs(n, m, seed):
    from torchquantum_gb300 import _lib

    rng = np.random.default_rng(seed)
    xs = [int(v) for v in rng.integers(0, 1 << n, size=m)]
    zs = [int(v) for v in rng.integers(0, 1 << n, size=m)]
    xs[0] = 0  # a diagonal string
    for group, c, r in _lib.coset_groups(xs, n):
        model, r2 = _coset_model(n, xs, zs, group, c)
        assert r2 == r and c + r == min(n, 13) and len(group) <= 8
        seen = np.zeros(1 << n, dtype=np.int64)
        for gidx, consts, rho in model:
            g = np.array(gidx)
            seen[g] += 1
            for s, j in enumerate(group):
                xsu, gam, _ = consts[s]
                for u in range(len(gidx)):
                    assert gidx[u ^ xsu] == gidx[u] ^ xs[j]  # partner on chip
                    assert (bin(gidx[u] & zs[j]).count("1") & 1) == (rho[s] ^ (bin(u & gam).count("1") & 1))
        assert (seen == 1).all()  # the cosets partition the row


@pytest.mark.parametrize("n,m,seed", [(6, 5, 10), (14, 9, 11)])
def test_coset_expvals_and_seed_match_the_oracle(n, m, seed):
    """Expvals and the backward seed assembled from the coset model (the kernel's sign
    bits: expvals ny >> 1, seed (ny & 1) ^ (ny >> 1)) equal the oracle's."""
    from torchquantum_gb300 import _lib

    rng = np.random.default_rng(seed)
    strings = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(m)]
    masks = [O.pauli_masks(p, n) for p in strings]
    xs, zs = [x for x, _, _ in masks], [z for _, z, _ in masks]
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    coef = rng.normal(size=m)
    ev = np.zeros(m)
    seed_out = np.zeros(1 << n, dtype=np.complex128)
    for group, c, r in _lib.coset_groups(xs, n):
        model, _ = _coset_model(n, xs, zs, group, c)
        for gidx, consts, rho in model:
            g = np.array(gidx)
            stage = psi[g]
            for s, j in enumerate(group):
                xsu, gam, _ = consts[s]
                ny = bin(xs[j] & zs[j]).count("1") & 3
                for u in range(len(gidx)):
                    pb = rho[s] ^ (bin(u & gam).count("1") & 1)
                    w = np.conj(stage[u]) * stage[u ^ xsu]
                    part = w.imag if ny & 1 else w.real
                    ev[j] += part * (-1) ** (pb ^ (ny >> 1))
                    term = stage[u ^ xsu] * (1j if ny & 1 else 1)
                    seed_out[g[u]] += coef[j] * (-1) ** (pb ^ (ny & 1) ^ (ny >> 1)) * term
    want = np.array([O.expval_pauli(psi[None], p, n)[0] for p in strings])
    assert np.abs(ev - want).max() < 1e-9
    # the expval kernel's halved rule: per pair (u, u + 1) of stage coordinates, a string
    # with xs = 0 adds both |psi|^2 terms, xs = 1 adds twice the u-side term, any other xs
    # adds twice both terms when bit hb (the highest of xs) of u is clear, else nothing
    half = np.zeros(m)
    for group, c, r in _lib.coset_groups(xs, n):
        model, _ = _coset_model(n, xs, zs, group, c)
        for gidx, consts, rho in model:
            stage = psi[np.array(gidx)]
            for s, j in enumerate(group):
                xsu, gam, _ = consts[s]
                ny = bin(xs[j] & zs[j]).count("1") & 3
                hb = xsu.bit_length() - 1
                for u in range(0, len(gidx), 2):
                    pb = rho[s] ^ (bin(u & gam).count("1") & 1)
                    sgn0 = (-1) ** (pb ^ (ny >> 1))
                    sgn1 = sgn0 * (-1 if gam & 1 else 1)
                    if xsu == 0:
                        half[j] += sgn0 * abs(stage[u]) ** 2 + sgn1 * abs(stage[u + 1]) ** 2
                    elif xsu == 1:
                        w0 = np.conj(stage[u]) * stage[u + 1]
                        half[j] += 2 * sgn0 * (w0.imag if ny & 1 else w0.real)
                    elif not (u >> hb) & 1:
                        w0 = np.conj(stage[u]) * stage[u ^ xsu]
                        w1 = np.conj(stage[u + 1]) * stage[(u + 1) ^ xsu]
                        part = (w0.imag, w1.imag) if ny & 1 else (w0.real, w1.real)
                        half[j] += 2 * (sgn0 * part[0] + sgn1 * part[1])
    assert np.abs(half - want).max() < 1e-9
    want_seed = sum(cj * O.apply_pauli(psi[None], p, n)[0] for cj, p in zip(coef, strings))
    assert np.abs(seed_out - want_seed).max() < 1e-9
