"""The coarsest level's two cooperative launches, replayed on the CPU for the
grids the library is used on (no GPU needed).

Band Cholesky (pf_kernel, csrc/tp_cholesky.cu): the work items of the 151
non-chain CTAs (pf_plan's per-step counts, pf_item's decoding) stay inside the
flag arrays; every tile (I, J) receives the update of every step k that reaches
it, once, in step order (from the bulk items and the chain's own update of tile
(k+1, k+1)); and a replay in which each CTA takes its items in order and waits
on exactly the flags pf_wait_item / pf_chain wait on runs to the end -- so no
bounded wait in the kernel is ever the one that gives up by design.

Triangular solves (ps_solve_kernel): for ps_plan's row split (R rows per CTA,
P warps per row, mirrored rows ps_row_of, the paired warps of ps_warp_row),
every phase covers each row of its block once, each row's parts tile its
range, the staged segment fits the shared memory the plan reserves, every read
stays inside its array, the forward phase reads only earlier blocks' solution
and the backward phase only later rows'."""
import pytest

NSM = 152  # GB300


def coarse(nelx, nely, nelz, nl):
    """Order and half bandwidth of the coarsest operator (coarse_alloc)."""
    s = 1 << (nl - 1)
    nx, ny, nz = nelx // s + 1, nely // s + 1, nelz // s + 1
    n = 3 * nx * ny * nz
    bw = 3 * (nz * ny + ny + 1) + 2
    return n, max(1, min(bw, n - 1))


GRIDS = {  # the grids of the bench, the tests and smoke()
    "48x24x24_l3": coarse(48, 24, 24, 3), "128x64x64_l4": coarse(128, 64, 64, 4),
    "256x128x128_l4": coarse(256, 128, 128, 4), "64x32x32_l4": coarse(64, 32, 32, 4),
    "64x64x64_l3": coarse(64, 64, 64, 3), "16x8x8_l3": coarse(16, 8, 8, 3), "narrow_200_150": (200, 150),
}


def pf_imax(n, bw, k):
    """Last tile row of step k's panel (k itself: no panel)."""
    if 32 * (k + 1) >= n:
        return k
    return min(n - 1, 32 * k + 31 + bw) // 32


@pytest.mark.parametrize("grid", list(GRIDS), ids=list(GRIDS))
def test_band_cholesky_schedule(grid):
    n, bw = GRIDS[grid]
    NT = (n + 31) // 32
    TS, off = 2, [0]
    for k in range(NT):
        T = pf_imax(n, bw, k) - k
        TS = max(TS, T + 2)
        off.append(off[-1] + ((T - 1) + T * (T + 1) // 2 - 1 if T >= 1 else 0))
    total, nbulk = off[-1], NSM - 1

    def item(g, k):
        while off[k + 1] <= g:
            k += 1
        idx = g - off[k]
        T = pf_imax(n, bw, k) - k
        prev = pf_imax(n, bw, k - 1) if k >= 1 else -1
        if idx < T - 1:  # panel tile (I, k)
            I = k + 2 + idx
            deps = [("f", k)] + ([("t", k, I - k, k)] if I <= prev else [])
            return k, ("S", k, I, None), deps, [("s", k, I - k)]
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

    # indices inside the flag arrays; every tile updated by every step that reaches it, once, in order
    upd = {}
    kk = 0
    for g in range(total):
        kk, (kind, k, I, J), _, _ = item(g, kk)
        assert 0 <= k < NT and I < NT
        if kind == "S":
            assert 2 <= I - k < TS
        else:
            assert k + 1 <= J <= I <= pf_imax(n, bw, k) and I - J < TS
            upd.setdefault((I, J), []).append(k)
    for k in range(NT):
        if pf_imax(n, bw, k) >= k + 1:
            upd.setdefault((k + 1, k + 1), []).append(k)  # the chain's own update
    for (I, J), ks in upd.items():
        assert ks == [k for k in range(NT) if J >= k + 1 and I <= pf_imax(n, bw, k)], (I, J)

    # replay: the chain in step order, each other CTA its items g = b, b + nbulk, ... in order
    done, tver = set(), {}

    def sat(d):
        return tver.get((d[1], d[2]), 0) >= d[3] if d[0] == "t" else d in done

    pos, kpos = list(range(nbulk)), [0] * nbulk
    k, ph, progress = 0, 0, True
    while progress:
        progress = False
        while k < NT:
            prev = k >= 1 and k + 1 <= pf_imax(n, bw, k - 1)
            if ph == 0:  # factor tile (k, k), release fdone[k]
                done.add(("f", k))
                progress = True
                if pf_imax(n, bw, k) < k + 1:
                    k = NT
                    break
                ph = 1
            if ph == 1:  # panel tile (k+1, k) after step k-1's update of it
                if prev and not sat(("t", k, 1, k)):
                    break
                done.add(("s", k, 1))
                ph, progress = 2, True
            if ph == 2:  # tile (k+1, k+1) after step k-1's update, then step k's
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


@pytest.mark.parametrize("grid", list(GRIDS), ids=list(GRIDS))
def test_band_cholesky_schedule_double_single(grid):
    """The double-single form of the factor (pf_chain_ds / pf_bulk_ds) takes
    the same items in the same round-robin order, but its chain waits
    differently: fdone[k] is released right after the factor is stored, and
    the panel solve waits for step k-1's updates of tiles (k+1,k) and
    (k+1,k+1) together. A replay with these waits runs to the end."""
    n, bw = GRIDS[grid]
    NT = (n + 31) // 32
    off = [0]
    for k in range(NT):
        T = pf_imax(n, bw, k) - k
        off.append(off[-1] + ((T - 1) + T * (T + 1) // 2 - 1 if T >= 1 else 0))
    total, nbulk = off[-1], NSM - 1

    def deps_of(g, k):
        while off[k + 1] <= g:
            k += 1
        idx = g - off[k]
        T = pf_imax(n, bw, k) - k
        prev = pf_imax(n, bw, k - 1) if k >= 1 else -1
        if idx < T - 1:
            I = k + 2 + idx
            return k, [("f", k)] + ([("t", k, I - k, k)] if I <= prev else []), [("s", k, I - k)]
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
        return k, deps, [("t", J, I - J, k + 1)]

    done, tver = set(), {}

    def sat(d):
        return tver.get((d[1], d[2]), 0) >= d[3] if d[0] == "t" else d in done

    pos, kpos = list(range(nbulk)), [0] * nbulk
    k, ph, progress = 0, 0, True
    while progress:
        progress = False
        while k < NT:
            prev = k >= 1 and k + 1 <= pf_imax(n, bw, k - 1)
            if ph == 0:  # factor tile (k, k), store it, release fdone[k]
                done.add(("f", k))
                progress = True
                if pf_imax(n, bw, k) < k + 1:
                    k = NT
                    break
                ph = 1
            if ph == 1:  # tiles (k+1, k) and (k+1, k+1) after step k-1's updates
                if prev and not (sat(("t", k, 1, k)) and sat(("t", k + 1, 0, k))):
                    break
                done.add(("s", k, 1))
                tver[(k + 1, 0)] = k + 1
                k, ph, progress = k + 1, 0, True
        for b in range(nbulk):
            while pos[b] < total:
                kpos[b], deps, outs = deps_of(pos[b], kpos[b])
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


def ps_warp_row(w, R, P):
    if R == 4:
        return ((w >> 1) if w < 4 else 3 - ((w - 4) >> 1)), w & 1
    return w // P, w % P


def ps_row_of(b, rl, G):
    return rl * G + ((G - 1 - b) if (rl & 1) else b)


@pytest.mark.parametrize("grid", list(GRIDS), ids=list(GRIDS))
def test_coarse_solve_phases(grid):
    n, bw = GRIDS[grid]
    nbs = min(min(768, max(512, 4 * NSM // 32 * 32)), (n + 31) // 32 * 32)  # coarse_alloc: 4 rows per SM
    nblk = (n + nbs - 1) // nbs
    R = 1
    while R < 8 and (nbs + R - 1) // R > NSM:
        R *= 2
    P = 8 // R
    G = (nbs + R - 1) // R
    assert G <= NSM
    seg = max((bw + P - 1) // P, (nbs + P - 1) // P)
    assert (2 * 8 * seg + 8 * 8) * 8 <= 200 * 1024  # the plan's shared-memory cap
    band, lsz, dsz = n * (bw + 1) + 1, nblk * nbs * bw, nblk * nbs * nbs
    # the rows of a CTA pair short with long: a bijection onto 0 .. R*G-1
    assert sorted(ps_row_of(b, rl, G) for b in range(G) for rl in range(R)) == list(range(R * G))
    for w in range(8):
        rl, p = ps_warp_row(w, R, P)
        assert 0 <= rl < R and 0 <= p < P
    assert sorted(ps_warp_row(w, R, P) for w in range(8)) == [(r, q) for r in range(R) for q in range(P)]
    nph, nf = 4 * nblk - 2, 2 * nblk - 1
    for h in range(nph):
        if h < nf:
            k, kind = (h + 1) // 2, ("FA" if h & 1 else "FB")
        else:
            q = h - nf
            k, kind = nblk - 1 - (q + 1) // 2, ("BA" if q & 1 else "BB")
        assert 0 <= k < nblk and (kind != "FA" or k > 0) and (kind != "BA" or k < nblk - 1)
        b0 = k * nbs
        s = min(nbs, n - b0)
        seen = {}
        for cta in range(G):
            for w in range(8):
                rl, p = ps_warp_row(w, R, P)
                i = ps_row_of(cta, rl, G)
                if i >= s:
                    continue
                if kind == "FA":
                    m, mlim, voff, lo, hi = (k * nbs + i) * bw, lsz, b0 - bw, max(0, bw - b0, i), bw
                elif kind == "FB":
                    m, mlim, voff, lo, hi = (k * nbs + i) * nbs, dsz, b0, 0, i + 1
                elif kind == "BA":
                    rr, b1 = b0 + i, min(n, b0 + nbs)
                    m, mlim, voff, lo, hi = rr * bw, band, 0, b1, min(n - 1, rr + bw) + 1
                else:
                    m, mlim, voff, lo, hi = (k * nbs + i) * nbs, dsz, b0, i, s
                ln = max(0, hi - lo)
                cs = (ln + P - 1) // P
                a0, a1 = lo + p * cs, min(hi, lo + p * cs + cs)
                seen.setdefault(i, []).append((a0, a1) if a1 > a0 else None)
                if a1 <= a0:
                    continue
                assert a1 - a0 <= seg
                assert 0 <= m + a0 and m + a1 - 1 < mlim, (kind, k, i)
                assert 0 <= voff + a0 and voff + a1 - 1 < n, (kind, k, i)
                if kind == "FA":
                    assert voff + a1 - 1 < b0  # earlier blocks only
                if kind == "BA":
                    assert voff + a0 >= min(n, b0 + nbs)  # later rows only
        assert sorted(seen) == list(range(s)), (kind, k)
        for i, parts in seen.items():
            assert len(parts) == P
            spans = sorted(x for x in parts if x)
            for (a, b), (c, _) in zip(spans, spans[1:]):
                assert b == c  # the parts tile the row's range without overlap
