"""CPU model of the cluster kernel's data movement (``csrc/cluster.cu``).

The single-lattice cluster kernel keeps a slab of rows per CTA in shared
memory in the resident kernel's band layout and exchanges halo rows through
parity-double-buffered halo areas and, between CTAs, remote stores into the
neighbours' "row above" / "row below" slots, with one cluster barrier per
generation.  This test replays that protocol lane by lane on the CPU -- warps
in lockstep (the row shuffles read the neighbouring lanes' words of the same
step), one shared array per CTA, remote stores into the other CTAs' arrays,
the launch shapes ``xk_life_cluster_config`` picks -- and checks that

* every shared-memory index lies inside the allocation the host sizes
  (``cluster_words``), and the slab never reaches into the halo area;
* every halo or slot word that generation g reads was written for generation
  g (by the publication before the first generation, or by generation g - 1);
* the lattice after the run equals a plain Life run (torus and static border).

The layout arithmetic restates ``life_word.cuh`` (``xk_resident_plan``,
``xk_res_at``, ``xk_res_lat_words``) and ``cluster.cu``; the Life rule itself is
evaluated bit by bit here (the kernel's rule table is covered by the GPU
tests).
"""
import numpy as np
import pytest

M32 = 0xFFFFFFFF


def plan(wpr, H, threads):
    P = 1
    while P < wpr:
        P <<= 1
    gpw = 32 // P
    groups = min((threads // 32) * gpw, H)
    L = (H + groups - 1) // groups
    return dict(P=P, gpw=gpw, G=groups, L=L, nb=(H + L - 1) // L)


def at(p, b, i, jj):
    return ((b // p["gpw"]) * p["L"] + i) * 32 + (b % p["gpw"]) * p["P"] + jj


def lat_words(p):
    return p["L"] * ((p["G"] + p["gpw"] - 1) // p["gpw"]) * 32


def cluster_words(wpr, R, threads):
    p = plan(wpr, R, threads)
    return lat_words(p) + 4 * p["G"] * wpr + 4 * wpr


def config(W, H, C, band):
    """xk_life_cluster_config without the device queries."""
    wpr = (W + 31) // 32
    if wpr > 32 or C < 2 or C > 16 or H < C:
        return None
    rows = (H + C - 1) // C
    Cr = (H + rows - 1) // rows
    if Cr < 2:
        return None
    P = 1
    while P < wpr:
        P <<= 1
    groups = (rows + band - 1) // band
    th = max(32, min(1024, ((P * groups + 31) // 32) * 32))
    return Cr, rows, th


def life_ref(grid, gens, torus, border):
    g = grid.copy()
    H, W = g.shape
    for _ in range(gens):
        if torus:
            n = sum(np.roll(np.roll(g, dy, 0), dx, 1)
                    for dy in (-1, 0, 1) for dx in (-1, 0, 1) if (dy, dx) != (0, 0))
        else:
            pad = np.full((H + 2, W + 2), border, np.int64)
            pad[1:-1, 1:-1] = g
            n = sum(pad[1 + dy:1 + dy + H, 1 + dx:1 + dx + W]
                    for dy in (-1, 0, 1) for dx in (-1, 0, 1) if (dy, dx) != (0, 0))
        g = ((n == 3) | ((n == 2) & (g == 1))).astype(np.int64)
    return g


class Smem:
    """One CTA's shared memory: values plus the generation each word was
    written for."""

    def __init__(self, n):
        self.v = [0] * n
        self.gen = [None] * n

    def rd(self, a):
        assert 0 <= a < len(self.v), ("shared read out of bounds", a, len(self.v))
        return self.v[a]

    def wr(self, a, x, gen):
        assert 0 <= a < len(self.v), ("shared write out of bounds", a, len(self.v))
        self.v[a] = x & M32
        self.gen[a] = gen


def next_word(rows, centre):
    """B3/S23 for the 32 cells of a word from the (L, C, R) vectors of the
    rows above, at and below."""
    out = 0
    for b in range(32):
        n = sum((x >> b) & 1 for r, row in enumerate(rows) for k, x in enumerate(row)
                if not (r == 1 and k == 1))
        if n == 3 or (n == 2 and (centre >> b) & 1):
            out |= 1 << b
    return out


def run(W, H, C_want, band, gens, torus, border, seed):
    cfg = config(W, H, C_want, band)
    assert cfg is not None
    C, R, threads = cfg
    wpr = (W + 31) // 32
    rlast = W - 32 * (wpr - 1)
    lastmask = M32 if rlast == 32 else (1 << rlast) - 1
    bfill = M32 if border else 0
    edge = bfill & 1
    grid = (np.random.RandomState(seed).random_sample((H, W)) < 0.45).astype(np.int64)
    words = [sum(int(grid[y, 32 * jw + k]) << k for k in range(32) if 32 * jw + k < W)
             for y in range(H) for jw in range(wpr)]
    pw = plan(wpr, R, threads)
    halo_at = lat_words(pw)
    slot_at = halo_at + 4 * pw["G"] * wpr
    hwords = 2 * pw["G"] * wpr
    sm = [Smem(cluster_words(wpr, R, threads)) for _ in range(C)]
    ctas = []
    for c in range(C):
        r0 = c * R
        Rc = min(H, r0 + R) - r0
        p = plan(wpr, Rc, threads)
        for w in range(Rc * wpr):
            y, jj = divmod(w, wpr)
            b, i = divmod(y, p["L"])
            assert at(p, b, i, jj) < halo_at
            sm[c].wr(at(p, b, i, jj), words[r0 * wpr + w], "load")
        lanes = []
        for t in range(threads):
            lane, warp = t & 31, t >> 5
            q, j = divmod(lane, p["P"])
            band_ = warp * p["gpw"] + q
            bc = band_ if band_ < p["nb"] else p["nb"] - 1
            jc = j if j < wpr else wpr - 1
            y0 = bc * p["L"]
            last = wpr - 1
            lshift = 31 if jc > 0 else rlast - 1
            d = dict(active=band_ < p["nb"] and j < wpr, band=band_, bc=bc, j=j, jc=jc,
                     y0=y0, n=min(Rc, y0 + p["L"]) - y0,
                     src_l=q * p["P"] + (jc - 1 if jc > 0 else last),
                     src_r=q * p["P"] + (jc + 1 if jc < last else 0),
                     lshift=lshift, lpre=31 - lshift, top=rlast - 1 if jc == last else 31,
                     outmask=lastmask if jc == last else M32,
                     use_le=(not torus) and jc == 0, use_re=(not torus) and jc == last,
                     first=bc == 0, lastb=bc == p["nb"] - 1, wp=at(p, bc, 0, jc))
            d["top_off"] = (not torus) and c == 0 and d["first"]
            d["bot_off"] = (not torus) and c == C - 1 and d["lastb"]
            lanes.append(d)
        ctas.append(dict(c=c, r0=r0, Rc=Rc, p=p, lanes=lanes,
                         up=c - 1 if c > 0 else C - 1, dn=c + 1 if c + 1 < C else 0))

    def vec(d, w, l, r):
        if torus:
            left = ((w << 1) | (((l << d["lpre"]) & M32) >> 31)) & M32
            right = (w >> 1) | ((r << d["top"]) & M32 & (1 << d["top"]))
        else:
            lb = edge if d["use_le"] else (l >> d["lshift"]) & 1
            rb = edge if d["use_re"] else r & 1
            left = ((w << 1) | lb) & M32
            right = (w >> 1) | (rb << d["top"])
        return (left, w, right & M32)

    def publish(ct, d, par, i, w, gen):
        # a band's first row to its halo (and, for the slab's first band, to
        # the CTA above's "row below" slot); its last row likewise downwards
        if not d["active"]:
            return
        c, p = ct["c"], ct["p"]
        if i == 0:
            sm[c].wr(halo_at + par * hwords + (d["band"] * 2 + 0) * wpr + d["j"], w, gen)
            if d["band"] == 0:
                sm[ct["up"]].wr(slot_at + (par * 2 + 1) * wpr + d["j"], w, gen)
        if i == d["n"] - 1:
            sm[c].wr(halo_at + par * hwords + (d["band"] * 2 + 1) * wpr + d["j"], w, gen)
            if d["band"] == p["nb"] - 1:
                sm[ct["dn"]].wr(slot_at + (par * 2 + 0) * wpr + d["j"], w, gen)

    for ct in ctas:
        for d in ct["lanes"]:
            publish(ct, d, 0, 0, sm[ct["c"]].rd(d["wp"]), 0)
            publish(ct, d, 0, d["n"] - 1, sm[ct["c"]].rd(d["wp"] + 32 * (d["n"] - 1)), 0)
    for gen in range(gens):
        par = gen & 1
        for ct in ctas:                      # the barrier: every CTA sees generation gen
            S, p = sm[ct["c"]], ct["p"]
            hp = halo_at + par * hwords
            for w0 in range(0, threads, 32):
                ls = ct["lanes"][w0:w0 + 32]

                def fresh(a, off):
                    v = S.rd(a)
                    assert off or S.gen[a] == gen, ("stale halo", gen, S.gen[a])
                    return v

                wu = [fresh(slot_at + (par * 2) * wpr + d["jc"] if d["first"]
                            else hp + ((d["bc"] - 1) * 2 + 1) * wpr + d["jc"], d["top_off"])
                      for d in ls]
                wl = [fresh(slot_at + (par * 2 + 1) * wpr + d["jc"] if d["lastb"]
                            else hp + ((d["bc"] + 1) * 2) * wpr + d["jc"], d["bot_off"])
                      for d in ls]

                def vecs(ws, off):
                    return [(bfill,) * 3 if off[k] else vec(d, ws[k], ws[d["src_l"]], ws[d["src_r"]])
                            for k, d in enumerate(ls)]

                vu = vecs(wu, [d["top_off"] for d in ls])
                cm = [S.rd(d["wp"]) for d in ls]
                vm = vecs(cm, [False] * 32)
                for i in range(p["L"]):
                    edge_row = [i + 1 >= d["n"] for d in ls]
                    wd = [wl[k] if edge_row[k] else S.rd(d["wp"] + 32 * (i + 1))
                          for k, d in enumerate(ls)]
                    vd = vecs(wd, [edge_row[k] and d["bot_off"] for k, d in enumerate(ls)])
                    for k, d in enumerate(ls):
                        if d["active"] and i < d["n"]:
                            out = next_word((vu[k], vm[k], vd[k]), cm[k]) & d["outmask"]
                            assert d["wp"] + 32 * i < halo_at
                            S.wr(d["wp"] + 32 * i, out, ("lattice", gen))
                            publish(ct, d, par ^ 1, i, out, gen + 1)
                    vu, vm, cm = vm, vd, wd
    got = np.zeros((H, W), np.int64)
    for ct in ctas:
        p = ct["p"]
        for w in range(ct["Rc"] * wpr):
            y, jj = divmod(w, wpr)
            b, i = divmod(y, p["L"])
            word = sm[ct["c"]].rd(at(p, b, i, jj))
            for k in range(min(32, W - 32 * jj)):
                got[ct["r0"] + y, 32 * jj + k] = (word >> k) & 1
    return got, life_ref(grid, gens, torus, border)


@pytest.mark.parametrize("W,H,C,band", [(64, 33, 16, 2), (33, 17, 4, 5), (100, 40, 8, 4),
                                        (1, 9, 2, 2), (32, 2, 2, 1), (7, 70, 16, 5),
                                        (96, 45, 8, 3), (40, 64, 2, 4), (64, 100, 2, 1)])
@pytest.mark.parametrize("torus,border", [(True, 0), (False, 0), (False, 1)])
def test_cluster_halo_protocol(W, H, C, band, torus, border):
    got, want = run(W, H, C, band, 3, torus, border, W * 7 + H)
    assert np.array_equal(got, want)


# ---------------------------------------------------------------------------
# The neighbour form (P2P): CTAs wait only for their two neighbours' rows on
# mbarriers, and run generations at their own pace.  The model below replays
# that protocol with the CTAs (and the first and last band of each, which are
# different lanes and wait and send independently) interleaved in a random
# order, with the hardware's mbarrier semantics (a phase completes after the
# expected arrivals; a parity wait passes while the barrier's current phase
# parity differs from the one asked for), and checks that
#
# * every phase of every mbarrier completes with exactly 2 wpr arrivals, all
#   of them for the generation that phase belongs to (none of the next
#   generation's arrivals is counted early);
# * a wait passes only once the phase of its own generation has completed,
#   never two phases later (parity aliasing);
# * every slot word a band reads was written for the generation reading it,
#   and no slot word is overwritten before its reader has read it;
# * every CTA finishes (no wait is left that nothing will satisfy).

class Mbar:
    def __init__(self, expected):
        self.expected, self.pending, self.parity, self.done, self.tags = expected, expected, 0, 0, []

    def arrive(self, tag):
        self.tags.append(tag)
        self.pending -= 1
        assert self.pending >= 0
        if self.pending == 0:
            assert len(set(self.tags)) == 1, ("arrivals of several generations in one phase", self.tags)
            self.done += 1
            self.parity ^= 1
            self.pending, self.tags = self.expected, []

    def passes(self, parity):
        return self.parity != parity


def run_p2p(C, nb, wpr, gens, seed):
    rng = np.random.RandomState(seed)
    bars = [[Mbar(2 * wpr), Mbar(2 * wpr)] for _ in range(C)]
    # slot [cta][parity][above/below]: (generation tag, read since written)
    slot = {}
    agents = []
    for c in range(C):
        kinds = [("first", "last")] if nb == 1 else [("first",), ("last",)]
        for roles in kinds:
            agents.append(dict(c=c, roles=roles, gen=0, step="top"))
    up = [c - 1 if c > 0 else C - 1 for c in range(C)]
    dn = [c + 1 if c + 1 < C else 0 for c in range(C)]

    def send(c, role, g):
        # rows computed in generation g - 1 (or loaded, g = 0) for generation g
        par = g & 1
        tgt, side = (up[c], 1) if role == "first" else (dn[c], 0)
        key = (tgt, par, side)
        if key in slot:
            tag, read = slot[key]
            assert read, ("slot overwritten before it was read", key, tag, g)
        slot[key] = (g, False)
        for _ in range(wpr):
            bars[tgt][par].arrive(g)

    for c in range(C):                         # publication after the first cluster barrier
        for role in ("first", "last"):
            send(c, role, 0)
    for _ in range(100000):
        live = [a for a in agents if a["gen"] < gens]
        if not live:
            return True
        ready = []
        for a in live:
            g, c = a["gen"], a["c"]
            if a["step"] == "top":
                # __syncthreads_or at the top of generation g: released when
                # every band of the CTA has arrived there
                if all(b["gen"] == g and b["step"] == "top" for b in agents if b["c"] == c):
                    ready.append(a)
            elif a["step"] == "wait":
                if bars[c][g & 1].passes((g >> 1) & 1):
                    ready.append(a)
            else:
                ready.append(a)
        assert ready, "deadlock"
        a = ready[rng.randint(len(ready))]
        g, c = a["gen"], a["c"]
        if a["step"] == "top":
            for b in agents:                   # the barrier releases the whole CTA
                if b["c"] == c:
                    b["step"] = "wait"
        elif a["step"] == "wait":
            assert bars[c][g & 1].done == (g >> 1) + 1, ("wait passed on another phase", g)
            a["step"] = "read"
        elif a["step"] == "read":
            for role in a["roles"]:
                key = (c, g & 1, 0 if role == "first" else 1)
                tag, _ = slot[key]
                assert tag == g, ("slot of another generation", key, tag, g)
                slot[key] = (tag, True)
            a["step"] = "send"
        else:
            if g + 1 < gens:                   # the last generation sends nothing
                for role in a["roles"]:
                    send(c, role, g + 1)
            a["gen"], a["step"] = g + 1, "top"
    raise AssertionError("no progress")


@pytest.mark.parametrize("C", [2, 3, 4, 16])
@pytest.mark.parametrize("nb", [1, 2, 5])
def test_neighbour_form_protocol(C, nb):
    for seed in range(12):
        assert run_p2p(C, nb, wpr=3, gens=9, seed=seed * 31 + C * 7 + nb)


def test_neighbour_form_mbarriers_fit_the_allocation():
    """The two mbarriers sit 8-byte aligned after the slab, halos and slots,
    inside the shared memory the host sizes."""
    for W, H, C, band in [(64, 33, 16, 2), (33, 17, 4, 1), (100, 40, 8, 4), (1, 9, 2, 2),
                          (1024, 1024, 16, 4), (512, 512, 16, 2), (7, 70, 16, 1)]:
        Cr, R, threads = config(W, H, C, band)
        wpr = (W + 31) // 32
        data = cluster_words(wpr, R, threads)
        total = ((data + 1) & ~1) + 4
        mbar_word = (data + 1) & ~1
        assert mbar_word % 2 == 0 and mbar_word >= data and mbar_word + 4 <= total


# ---------------------------------------------------------------------------
# The async form: the neighbour form's order of waits and sends, but each row
# word travels as an asynchronous remote store that lands some time later and
# then counts 4 bytes (here: one word) of the transaction count of the
# receiver's mbarrier of that parity.  The receiving CTA's thread 0 (a lane of
# its first band) arms that mbarrier once per phase, at the top of the
# generation that reads it, with one arrival expecting the 2 wpr words.  The
# model delivers the stores in flight in a random order, interleaved with the
# bands' steps, and checks that
#
# * a phase completes only with its arming and all 2 wpr words of its own
#   generation (a word that lands before the arming waits for it; none of the
#   next generation's words is counted early);
# * a wait passes only on the phase of its own generation;
# * a store never lands on a slot word its reader has not read yet, and every
#   slot word a band reads was written for the generation reading it;
# * nothing is left in flight when every CTA has finished.

class TxBar:
    def __init__(self, words):
        self.words, self.pending, self.tx, self.parity, self.done, self.tags = words, 1, 0, 0, 0, []

    def _check(self):
        if self.pending == 0 and self.tx == 0:
            assert len(set(self.tags)) == 1, ("several generations in one phase", self.tags)
            self.done += 1
            self.parity ^= 1
            self.pending, self.tags = 1, []

    def arm(self, gen):
        assert self.pending == 1, "armed twice in one phase"
        self.pending = 0
        self.tx += self.words
        self.tags.append(gen)
        self._check()

    def complete(self, gen):
        self.tx -= 1
        self.tags.append(gen)
        self._check()

    def passes(self, parity):
        return self.parity != parity


def run_async(C, nb, wpr, gens, seed):
    rng = np.random.RandomState(seed)
    bars = [[TxBar(2 * wpr), TxBar(2 * wpr)] for _ in range(C)]
    slot = {}              # (cta, parity, side, word) -> (generation tag, read since written)
    flight = []            # stores issued, not yet landed
    agents = []
    for c in range(C):
        kinds = [("first", "last")] if nb == 1 else [("first",), ("last",)]
        for roles in kinds:
            agents.append(dict(c=c, roles=roles, gen=0, step="arm" if "first" in roles else "top"))
    up = [c - 1 if c > 0 else C - 1 for c in range(C)]
    dn = [c + 1 if c + 1 < C else 0 for c in range(C)]

    def send(c, role, g):
        tgt, side = (up[c], 1) if role == "first" else (dn[c], 0)
        for j in range(wpr):
            flight.append((tgt, g & 1, side, j, g))

    def land(k):
        tgt, par, side, j, g = flight.pop(k)
        key = (tgt, par, side, j)
        if key in slot:
            tag, read = slot[key]
            assert read, ("store landed on a slot word not yet read", key, tag, g)
        slot[key] = (g, False)
        bars[tgt][par].complete(g)

    for c in range(C):
        for role in ("first", "last"):
            send(c, role, 0)
    for _ in range(200000):
        live = [a for a in agents if a["gen"] < gens]
        if not live:
            assert not flight, "stores still in flight at the end"
            return True
        ready = []
        for a in live:
            g, c = a["gen"], a["c"]
            if a["step"] == "top":
                if all(b["gen"] == g and b["step"] == "top" for b in agents if b["c"] == c):
                    ready.append(a)
            elif a["step"] == "wait":
                if bars[c][g & 1].passes((g >> 1) & 1):
                    ready.append(a)
            else:
                ready.append(a)
        choices = len(ready) + len(flight)
        assert choices, "deadlock"
        k = rng.randint(choices)
        if k >= len(ready):
            land(k - len(ready))
            continue
        a = ready[k]
        g, c = a["gen"], a["c"]
        if a["step"] == "arm":
            bars[c][g & 1].arm(g)
            a["step"] = "top"
        elif a["step"] == "top":
            for b in agents:
                if b["c"] == c:
                    b["step"] = "wait"
        elif a["step"] == "wait":
            assert bars[c][g & 1].done == (g >> 1) + 1, ("wait passed on another phase", g)
            a["step"] = "read"
        elif a["step"] == "read":
            for role in a["roles"]:
                for j in range(wpr):
                    key = (c, g & 1, 0 if role == "first" else 1, j)
                    tag, _ = slot[key]
                    assert tag == g, ("slot of another generation", key, tag, g)
                    slot[key] = (tag, True)
            a["step"] = "send"
        else:
            if g + 1 < gens:
                for role in a["roles"]:
                    send(c, role, g + 1)
            a["gen"] = g + 1
            a["step"] = "arm" if "first" in a["roles"] else "top"
    raise AssertionError("no progress")


@pytest.mark.parametrize("C", [2, 3, 4, 16])
@pytest.mark.parametrize("nb", [1, 2, 5])
def test_async_form_protocol(C, nb):
    for seed in range(12):
        assert run_async(C, nb, wpr=3, gens=9, seed=seed * 37 + C * 5 + nb)
