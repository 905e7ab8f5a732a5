"""The dissected coarsest-level factor (tp_set_coarse_order(c, 1), the
default), checked on the CPU (no GPU needed).

1. A numpy model of the composite layout and of the launch sequence, written
   with the index arithmetic of csrc/tp_cholesky.cu: nd_layout's views, pads
   and origins, nd_scatter_kernel's placement (natural order for part A and
   the separator S, mirrored plane order for part B), the partial factors of
   the views A and B, nd_schur_kernel's sum of their trailing blocks, S's
   factor, the block inverses and block rows (dinv_kernel, lrow_kernel), the
   tails' rows, and the solve: the forward phases of both views
   (ps_solve_kernel's FA / FB rows), nd_couple_kernel, S's forward and
   backward phases, nd_tails_kernel, the backward phases with tails (BA of
   every block, the last included) and the gather / scatter through nd_map;
   with both halves in every phase and with the halves swept in turn (the
   form for bands too wide for a phase of both).
   On small grids with a random SPD operator of the coarse pattern (fixed
   rows and columns as the coarsest level has them) the composite solve
   equals a dense solve to rounding, with equal and unequal halves and with
   blocks narrower than the band.
2. The partial factors' schedule: pf_kernel runs NT = own / 32 steps of a
   view's band, on its share of the CTAs (nd_split). Replayed as in
   test_coarse_schedule.py for the views of the grids the library is used on
   (three CTAs per SM in double-single, two in FP64, split between the
   views in proportion to their rows):
   every flag index stays inside its array (tver has a row per tile of the
   view, the trailing block's tiles included), every tile of the trailing
   block receives every step's update once and in order (the last one of
   tile (NT, NT) from the chain, which then stores it), and the replay runs
   to the end with both chains' waits (FP64 and double-single)."""
import numpy as np
import pytest

NSM = 152  # GB300


def layout(nx, ny, nz, nbs):
    """nd_layout: separator plane, pads, own rows, view origins, blocks."""
    xs = (nx - 1) // 2
    plane = 3 * ny * nz
    na, nb = plane * xs, plane * (nx - 1 - xs)
    pad = [(32 - na % 32) % 32, (32 - nb % 32) % 32]
    own = [pad[0] + na, pad[1] + nb, plane]
    org = [0, own[0] + plane, own[0] + plane + own[1] + plane]
    nblk = [(o + nbs - 1) // nbs for o in own]
    bw = 3 * (nz * ny + ny + 1) + 2
    return dict(xs=xs, ns=plane, pad=pad, own=own, org=org, ntot=org[2] + plane, nblk=nblk, bw=bw)


def composite_solve(nx, ny, nz, lim, nbs, seed, sequential=False):
    rng = np.random.default_rng(seed)
    nn, n = nx * ny * nz, 3 * nx * ny * nz
    Ly = layout(nx, ny, nz, nbs)
    bw, ns, pad, own, org, ntot, nblk, xs = (Ly[k] for k in ("bw", "ns", "pad", "own", "org", "ntot", "nblk", "xs"))

    def node(i, k, j):
        return (i * nz + k) * ny + j

    # a random SPD operator with the coarse level's node couplings and boundary rows
    K = np.zeros((n, n))
    for a in range(nn):
        i, k, j = a // (ny * nz), (a // ny) % nz, a % ny
        for di in (-1, 0, 1):
            for dk in (-1, 0, 1):
                for dj in (-1, 0, 1):
                    ii, kk, jj = i + di, k + dk, j + dj
                    if 0 <= ii < nx and 0 <= kk < nz and 0 <= jj < ny and node(ii, kk, jj) < a:
                        b = node(ii, kk, jj)
                        blk = rng.uniform(-1, 1, (3, 3))
                        K[3 * a:3 * a + 3, 3 * b:3 * b + 3] = blk
                        K[3 * b:3 * b + 3, 3 * a:3 * a + 3] = blk.T
    K += np.diag(np.abs(K).sum(1) + 1.0)
    for k in range(nz):
        for j in range(ny):
            if j < lim or j >= ny - lim:
                for c in range(3):
                    f = 3 * node(0, k, j) + c
                    K[f, :] = 0.0
                    K[:, f] = 0.0
                    K[f, f] = 1.0

    # nd_scatter_kernel: the natural lower entries placed in the views' bands
    band = np.zeros(ntot * (bw + 1) + 1)

    def pos_b(p, k, j, c):  # nd_pos_b
        return pad[1] + 3 * (((nx - 1 - p) * nz + k) * ny + j) + c

    for t in range(pad[0]):
        band[t * bw + t] = 1.0
    for t in range(pad[1]):
        band[(org[1] + t) * bw + org[1] + t] = 1.0
    for a in range(nn):
        i, k, j = a // (ny * nz), (a // ny) % nz, a % ny
        for m in range(14):
            mi, mk, mj = i + m // 9 - 1, k + (m // 3) % 3 - 1, j + m % 3 - 1
            if not (0 <= mi < nx and 0 <= mk < nz and 0 <= mj < ny):
                continue
            b = node(mi, mk, mj)
            for c in range(3):
                for d in range(3):
                    r, col = 3 * a + c, 3 * b + d
                    if col > r or r - col > bw:
                        continue
                    if i <= xs:
                        band[(col + pad[0]) * bw + r + pad[0]] = K[r, col]
                    else:
                        pr, pc = pos_b(i, k, j, c), pos_b(mi, mk, mj, d)
                        assert abs(pr - pc) <= bw
                        band[(org[1] + min(pr, pc)) * bw + org[1] + max(pr, pc)] = K[r, col]

    # nd_map: a bijection of the own and S rows onto the natural rows
    mp = -np.ones(ntot, np.int64)
    mp[pad[0]:own[0]] = np.arange(own[0] - pad[0])
    for p in range(xs + 1, nx):
        for k in range(nz):
            for j in range(ny):
                for q in range(3):
                    mp[org[1] + pos_b(p, k, j, q)] = 3 * node(p, k, j) + q
    mp[org[2]:] = xs * ns + np.arange(ns)
    assert np.array_equal(np.sort(mp[mp >= 0]), np.arange(n))

    def nview(v):
        return own[v] + ns if v < 2 else ns

    def dense(v):
        o, nv = org[v], nview(v)
        M = np.zeros((nv, nv))
        for c in range(nv):
            for r in range(c, min(nv, c + bw + 1)):
                M[r, c] = band[(o + c) * bw + o + r]
        return M

    def store(v, M):
        o, nv = org[v], nview(v)
        for c in range(nv):
            for r in range(c, min(nv, c + bw + 1)):
                band[(o + c) * bw + o + r] = M[r, c]

    # partial factors: own rows eliminated, the trailing block keeps its updates
    for v in range(2):
        M = dense(v)
        M = np.tril(M) + np.tril(M, -1).T
        o = own[v]
        L11 = np.linalg.cholesky(M[:o, :o])
        L21 = np.linalg.solve(L11, M[o:, :o].T).T
        out = np.zeros_like(M)
        out[:o, :o], out[o:, :o], out[o:, o:] = L11, L21, M[o:, o:] - L21 @ L21.T
        store(v, np.tril(out))
    for jj in range(ns):  # nd_schur_kernel
        for ii in range(jj, ns):
            band[(org[2] + jj) * bw + org[2] + ii] = (band[(own[0] + jj) * bw + own[0] + ii] +
                                                     band[(org[1] + own[1] + jj) * bw + org[1] + own[1] + ii])
    MS = dense(2)
    store(2, np.linalg.cholesky(np.tril(MS) + np.tril(MS, -1).T))

    def bget(v, r, c):
        return band[(org[v] + c) * bw + org[v] + r] if 0 <= r - c <= bw else 0.0

    D, LR = {}, {}
    for v in range(3):
        for blk in range(nblk[v]):
            b0 = blk * nbs
            s = min(nbs, own[v] - b0)
            Lb = np.array([[bget(v, b0 + r, b0 + c) if c <= r else 0.0 for c in range(s)] for r in range(s)])
            D[v, blk] = np.zeros((nbs, nbs))
            D[v, blk][:s, :s] = np.linalg.inv(Lb)
            LR[v, blk] = np.array([[bget(v, b0 + i, b0 - bw + t) if b0 + i < own[v] and b0 - bw + t >= 0 else 0.0
                                    for t in range(bw)] for i in range(nbs)])
    tails = [np.array([[bget(v, own[v] + i, own[v] - bw + t) if own[v] - bw + t >= 0 else 0.0 for t in range(bw)]
                       for i in range(ns)]) for v in range(2)]

    b_nat = rng.uniform(-1, 1, n)
    rhs = np.where(mp >= 0, b_nat[np.maximum(mp, 0)], 0.0)  # nd_gather_kernel
    y, t, x = np.zeros(ntot), np.zeros(ntot), np.zeros(ntot)

    def phases(m, tail):  # ps_phase
        seq = [((h + 1) // 2, "FA" if h & 1 else "FB") for h in range(2 * m - 1)]
        for q in range(2 * m - (0 if tail else 1)):
            seq.append((m - 1 - q // 2, "BB" if q & 1 else "BA") if tail else
                       (m - 1 - (q + 1) // 2, "BA" if q & 1 else "BB"))
        return seq

    def run(views, m, tail, h0, h1):  # ps_row over the phases [h0, h1)
        seq = phases(m, tail)
        assert len(seq) == 4 * m - (1 if tail else 2)
        for k, kind in seq[h0:h1]:
            out = []
            for v in views:
                if k >= nblk[v]:
                    continue
                b0, vo = k * nbs, org[v]
                for i in range(min(nbs, own[v] - b0)):
                    if kind == "FA":
                        lo = max(0, bw - b0, i)
                        out.append((t, vo + b0 + i, rhs[vo + b0 + i] - LR[v, k][i, lo:] @ y[vo + b0 - bw + lo:vo + b0]))
                    elif kind == "FB":
                        vb = rhs if k == 0 else t
                        out.append((y, vo + b0 + i, D[v, k][i, :i + 1] @ vb[vo + b0:vo + b0 + i + 1]))
                    elif kind == "BA":
                        rr, b1 = b0 + i, min(own[v], b0 + nbs)
                        hi = min(nview(v) - 1, rr + bw) + 1
                        col = np.array([bget(v, e, rr) for e in range(b1, hi)])
                        out.append((t, vo + b0 + i, y[vo + b0 + i] - col @ x[vo + b1:vo + hi]))
                    else:
                        s = min(nbs, own[v] - b0)
                        vb = t if (tail or k != nblk[v] - 1) else y
                        out.append((x, vo + b0 + i, D[v, k][:s, i][i:] @ vb[vo + b0 + i:vo + b0 + s]))
            for arr, o, val in out:
                arr[o] = val

    m = max(nblk[0], nblk[1])

    def sweep(fwd):  # both halves in every phase, or one after the other (wide bands)
        if sequential:
            for v in (0, 1):
                mv = nblk[v]
                run([v], mv, 1, 0 if fwd else 2 * mv - 1, 2 * mv - 1 if fwd else 4 * mv - 1)
        else:
            run([0, 1], m, 1, 0 if fwd else 2 * m - 1, 2 * m - 1 if fwd else 4 * m - 1)

    sweep(True)
    for s in range(ns):  # nd_couple_kernel
        acc = 0.0
        for v in range(2):
            lo = max(s, bw - own[v])
            acc += tails[v][s, lo:] @ y[org[v] + own[v] - bw + lo:org[v] + own[v]]
        rhs[org[2] + s] -= acc
    run([2], nblk[2], 0, 0, 4 * nblk[2] - 2)
    for v in range(2):  # nd_tails_kernel
        x[org[v] + own[v]:org[v] + own[v] + ns] = x[org[2]:org[2] + ns]
    sweep(False)
    x_nat = np.zeros(n)
    x_nat[mp[mp >= 0]] = x[mp >= 0]  # nd_scatter_out_kernel
    ref = np.linalg.solve(K, b_nat)
    return np.linalg.norm(x_nat - ref) / np.linalg.norm(ref)


@pytest.mark.parametrize("sequential", [False, True], ids=["both_halves_per_phase", "halves_in_turn"])
@pytest.mark.parametrize("grid", [(9, 5, 5, 1, 64, 0), (8, 5, 5, 1, 96, 1), (11, 4, 6, 1, 128, 2)],
                         ids=["halves_4_4_bw_over_block", "halves_3_4", "halves_5_5"])
def test_composite_solve_model(grid, sequential):
    assert composite_solve(*grid, sequential=sequential) < 1e-12


def pf_imax(n, bw, k):
    if 32 * (k + 1) >= n:
        return k
    return min(n - 1, 32 * k + 31 + bw) // 32


def replay_partial(n, bw, NT, nbulk, ds):
    """pf_plan / pf_item / the chain of a factor of NT steps over n rows."""
    tiles = (n + 31) // 32
    TS, off = 2, [0]
    for k in range(NT):
        T = pf_imax(n, bw, k) - k
        TS = max(TS, T + 2)
        off.append(off[-1] + ((T - 1) + T * (T + 1) // 2 - 1 if T >= 1 else 0))
    total = off[-1]

    def item(g, k):
        while off[k + 1] <= g:
            k += 1
        idx = g - off[k]
        T = pf_imax(n, bw, k) - k
        prev = pf_imax(n, bw, k - 1) if k >= 1 else -1
        if idx < T - 1:
            I = k + 2 + idx
            return k, ("S", k, I, k), [("f", k)] + ([("t", k, I - k, k)] if I <= prev else []), [("s", k, I - k)]
        u = idx - (T - 1)
        if u < T - 1:
            I, J = k + 2 + u, k + 1
        else:
            u -= T - 1
            q = 0
            while (q + 1) * (q + 2) // 2 <= u:
                q += 1
            I, J = k + 2 + q, k + 2 + (u - q * (q + 1) // 2)
        deps = [("s", k, I - k)] + ([("s", k, J - k)] if J != I else []) + ([("t", J, I - J, k)] if I <= prev else [])
        return k, ("U", k, I, J), deps, [("t", J, I - J, k + 1)]

    upd, kk = {}, 0
    for g in range(total):
        kk, (kind, k, I, J), deps, _ = item(g, kk)
        assert 0 <= k < NT and I < tiles
        for d in deps:  # flag indices: fdone [NT], sdone [NT][TS], tver [tiles][TS]
            if d[0] == "f":
                assert d[1] < NT
            elif d[0] == "s":
                assert d[1] < NT and d[2] < TS
            else:
                assert d[1] < tiles and d[2] < TS
        if kind == "U":
            assert J < tiles and I - J < TS
            upd.setdefault((I, J), []).append(k)
    for k in range(NT):
        upd.setdefault((k + 1, k + 1), []).append(k)  # the chain's own update; (NT, NT) stored after the last
    for I in range(NT, tiles):
        for J in range(NT, I + 1):
            want = [k for k in range(NT) if J >= k + 1 and I <= pf_imax(n, bw, k)]
            assert upd.get((I, J), []) == want, (I, J)

    done, tver = set(), {}

    def sat(d):
        return tver.get((d[1], d[2]), 0) >= d[3] if d[0] == "t" else d in done

    pos, kpos = list(range(nbulk)), [0] * nbulk
    k, ph, progress = 0, 0, True
    while progress:
        progress = False
        while k < NT:
            prev = k >= 1 and k + 1 <= pf_imax(n, bw, k - 1)
            if ph == 0:
                done.add(("f", k))
                ph, progress = 1, True
                assert pf_imax(n, bw, k) >= k + 1  # a partial factor never runs out of band
            if ds:  # pf_chain_ds: tiles (k+1, k) and (k+1, k+1) together
                if prev and not (sat(("t", k, 1, k)) and sat(("t", k + 1, 0, k))):
                    break
                done.add(("s", k, 1))
                tver[(k + 1, 0)] = k + 1
                k, ph, progress = k + 1, 0, True
                continue
            if ph == 1:
                if prev and not sat(("t", k, 1, k)):
                    break
                done.add(("s", k, 1))
                ph, progress = 2, True
            if ph == 2:
                if prev and not sat(("t", k + 1, 0, k)):
                    break
                tver[(k + 1, 0)] = k + 1
                k, ph, progress = k + 1, 0, True
        for b in range(nbulk):
            while pos[b] < total:
                kpos[b], _, deps, outs = item(pos[b], kpos[b])
                if not all(sat(d) for d in deps):
                    break
                for o in outs:
                    if o[0] == "t":
                        tver[(o[1], o[2])] = o[3]
                    else:
                        done.add(o)
                pos[b] += nbulk
                progress = True
    assert k >= NT and all(p >= total for p in pos), "the schedule stalls"


def coarsest(nelx, nely, nelz, nl):
    s = 1 << (nl - 1)
    return nelx // s + 1, nely // s + 1, nelz // s + 1


GRIDS = {"256x128x128_l4": coarsest(256, 128, 128, 4), "128x64x64_l4": coarsest(128, 64, 64, 4),
         "64x64x64_l3": coarsest(64, 64, 64, 3), "60x32x32_l3": coarsest(60, 32, 32, 3),
         "48x24x24_l3": coarsest(48, 24, 24, 3)}


@pytest.mark.parametrize("ds", [False, True], ids=["fp64_chain", "ds_chain"])
@pytest.mark.parametrize("grid", list(GRIDS), ids=list(GRIDS))
def test_partial_factor_schedule(grid, ds):
    nx, ny, nz = GRIDS[grid]
    Ly = layout(nx, ny, nz, 608)
    own, ns, bw = Ly["own"], Ly["ns"], Ly["bw"]
    if own[0] // 32 < 2 or own[1] // 32 < 2 or ns < 64:
        pytest.skip("the natural band is used on this grid")
    grid = (3 if ds else 2) * NSM  # nd_grid: three CTAs per SM in double-single, two in FP64
    split = min(grid - 2, max(2, round(own[0] / (own[0] + own[1]) * grid)))  # nd_split
    for v, ncta in ((0, split), (1, grid - split)):
        replay_partial(own[v] + ns, bw, own[v] // 32, ncta - 1, ds)
