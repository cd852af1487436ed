"""The oracle's own problem builder — TEST INFRASTRUCTURE.

Builds the `nm_plan` record (the data layout of include/namics_gb300.h) that
oracle/scf_oracle.c reads, straight from Namics input text, without the
product's plan compiler or library.  The CPU legs of bench.py (the timed
CPU baseline and the reference arm) use it, so those legs load nothing but
oracle/liborc.so.  Scope: 1-gradient lattices (planar, cylindrical,
spherical; simple cubic or hexagonal), free / pinned / frozen segments,
linear and branched compositions, free / restricted / solvent molecules and
the DIIS keys of `newton`.  Anything else raises ValueError.

Each step restates the reference's own set-up (leermakers/Namics src/):
  lattice and curvature weights   lattice.cpp:267-601, LGrad1.cpp:16-70,
                                  LG1Planar.cpp:11-12
  boundary sources                lattice.cpp:94-196
  segment ranges, masks           segment.cpp:248-500, 855-879
  KSAM                            system.cpp generate_mask
  χ defaults and symmetry         system.cpp CheckChi_values
  compositions, block tree        molecule.cpp:1156-1275, 1282-1779
                                  (branched numbering reversed, :1740-1766)
  monomer list                    molecule.cpp:1785-1800
  iteration species               system.cpp:430-500 (MakeItsLists, IsUnique)
  newton defaults                 solve_scf.cpp:153-236
tests/test_oracle_plan.py pins it: the oracle gives bit-identical residuals
and solves on this record and on the product's for the same text.
"""
from __future__ import annotations

import ctypes as C
import re

import numpy as np

PIE = 3.14159265  # the reference's truncated pi (namics.cpp:49)
MIRROR, PERIODIC, SURFACE = 0, 1, 2
SEG_FREE, SEG_PINNED, SEG_FROZEN = 0, 1, 2
MOL_FREE, MOL_RESTRICTED, MOL_SOLVENT = 0, 1, 2

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


class Block(C.Structure):
    _fields_ = [("seg", C.c_int), ("molmon", C.c_int), ("length", C.c_int), ("s0", C.c_int),
                ("parent", C.c_int), ("mult", C.c_int), ("degeneracy", C.c_double),
                ("n_child", C.c_int), ("child0", C.c_int)]


class Molecule(C.Structure):
    _fields_ = [("freedom", C.c_int), ("pinned", C.c_int), ("n", C.c_double), ("theta", C.c_double),
                ("phibulk", C.c_double), ("chainlength", C.c_double), ("n_molmon", C.c_int),
                ("molmon_seg", ip), ("molmon_fraction", dp), ("n_blocks", C.c_int),
                ("blocks", C.POINTER(Block)), ("child_index", ip), ("n_store", C.c_int),
                ("charge", C.c_double), ("markov", C.c_int), ("bend", C.c_double * 3)]


class PlanRecord(C.Structure):
    _fields_ = [("gradients", C.c_int), ("MX", C.c_int), ("MY", C.c_int), ("MZ", C.c_int),
                ("geometry", C.c_int), ("lattice_type", C.c_int), ("stencil_full", C.c_int),
                ("bc", C.c_int * 6), ("JX", C.c_int), ("JY", C.c_int), ("M", C.c_int),
                ("lambda_", C.c_double), ("offset_first_layer", C.c_double), ("bond_length", C.c_double),
                ("volume", C.c_double), ("L", dp), ("lambda_1", dp), ("lambda0", dp), ("lambda1", dp),
                ("ksam", ip), ("n_seg", C.c_int), ("seg_name", C.POINTER(C.c_char_p)),
                ("seg_freedom", ip), ("seg_it", ip), ("seg_gmask", dp), ("seg_phi_frozen", dp),
                ("chi", dp), ("seg_valence", dp), ("seg_epsilon", dp), ("n_it", C.c_int), ("it_seg", ip),
                ("iv", C.c_int), ("charged", C.c_int), ("n_mol", C.c_int), ("mols", C.POINTER(Molecule)),
                ("solvent", C.c_int), ("neutralizer", C.c_int), ("diis_m", C.c_int),
                ("iterationlimit", C.c_int), ("max_norm", C.c_int), ("tolerance", C.c_double),
                ("deltamax", C.c_double), ("mol_name", C.POINTER(C.c_char_p)),
                ("search_mol", C.c_int), ("search_what", C.c_int), ("target_kind", C.c_int),
                ("target_mol", C.c_int), ("target_what", C.c_int), ("target_value", C.c_double),
                ("super_tolerance", C.c_double), ("super_deltamax", C.c_double),
                ("super_iterationlimit", C.c_int), ("scan_mol", C.c_int), ("scan_what", C.c_int),
                ("scan_n", C.c_int), ("scan_exponential", C.c_int), ("scan_start", C.c_double),
                ("scan_end", C.c_double), ("scan_step", C.c_double), ("save_memory", C.c_int),
                ("n_state", C.c_int), ("state_name", C.POINTER(C.c_char_p)), ("state_seg", ip),
                ("state_valence", dp), ("state_alphabulk", dp), ("state_it", ip), ("seg_nstate", ip),
                ("n_sp", C.c_int), ("chi_sp", dp), ("it_sp", ip), ("scan_state", C.c_int),
                ("scan_reaction", C.c_int)]


def _entries(text: str):
    """`class : name : key : value` lines of the first start block
    (input.cpp:3-78); the last occurrence of a key wins."""
    out = {}
    order: dict[str, list[str]] = {}
    for ln in text.splitlines():
        ln = ln.split("//")[0].strip()
        if not ln:
            continue
        if ln == "start":
            break
        p = [t.strip() for t in ln.split(":")]
        if len(p) < 4:
            raise ValueError(f"not 'class : name : key : value': {ln}")
        cls, name, key, val = p[0], p[1], p[2], ":".join(p[3:]).strip()
        out[(cls, name, key)] = val
        order.setdefault(cls, [])
        if name not in order[cls]:
            order[cls].append(name)
    return out, order


def _composition(comp: str, segidx: dict[str, int]):
    """Written segments of a linear or branched composition: a list of
    (segment, bonded-to) in written order, side chains `[...]` bonded to the
    segment written just before the bracket (molecule.cpp:1156-1275)."""
    nodes: list[list[int]] = []   # [seg, parent]
    written: list[int] = []

    def chain(s: str, attach: int) -> None:
        prev = attach
        pos = 0
        while pos < len(s):
            c = s[pos]
            if c == " ":
                pos += 1
            elif c == "[":
                depth, q = 0, pos
                while q < len(s):
                    depth += s[q] == "["
                    depth -= s[q] == "]"
                    if depth == 0:
                        break
                    q += 1
                if q >= len(s) or prev < 0:
                    raise ValueError("unbalanced '[' or side chain before any segment")
                chain(s[pos + 1:q], prev)
                pos = q + 1
            elif c == "(":
                m = re.match(r"\(([^()\[\]]+)\)(\d+)", s[pos:])
                if not m:
                    raise ValueError("only (name)count runs and [side chains] are restated here")
                name, cnt = m.group(1).strip(), int(m.group(2))
                if name not in segidx or cnt < 1:
                    raise ValueError(f"segment '{name}' is not a mon")
                for _ in range(cnt):
                    nodes.append([segidx[name], prev])
                    prev = len(nodes) - 1
                    written.append(prev)
                pos += m.end()
            else:
                raise ValueError(f"unexpected '{c}' in composition")

    chain(comp, -1)
    return nodes, written


def _blocks(nodes, root):
    """Rooted tree -> blocks (maximal runs of one segment type with one child
    each), numbered in post-order so children come first and the root block
    last; children in written order."""
    n = len(nodes)
    adj = [[] for _ in range(n)]
    for i, (_, p) in enumerate(nodes):
        if p >= 0:
            adj[i].append(p)
            adj[p].append(i)
    par = [-2] * n
    par[root] = -1
    order = [root]
    for u in order:
        for v in adj[u]:
            if par[v] == -2:
                par[v] = u
                order.append(v)
    if len(order) != n:
        raise ValueError("composition is not connected")
    ch = [[] for _ in range(n)]
    for i in range(n):
        if par[i] >= 0:
            ch[par[i]].append(i)
    seg = [s for s, _ in nodes]
    tb, blk_of = [], [-1] * n
    for i in range(n):
        if len(ch[i]) == 1 and seg[ch[i][0]] == seg[i]:
            continue  # not the far end of a run
        run, cur = [i], i
        while par[cur] >= 0 and len(ch[par[cur]]) == 1 and seg[par[cur]] == seg[i]:
            cur = par[cur]
            run.append(cur)
        for k in run:
            blk_of[k] = len(tb)
        tb.append((seg[i], run, par[cur]))
    nb = len(tb)
    bpar = [blk_of[t[2]] if t[2] >= 0 else -1 for t in tb]
    bch = [[] for _ in range(nb)]
    for b in range(nb):
        if bpar[b] >= 0:
            bch[bpar[b]].append(b)
    post, stack = [], [[blk_of[root], 0]]
    while stack:
        top = stack[-1]
        if top[1] < len(bch[top[0]]):
            stack.append([bch[top[0]][top[1]], 0])
            top[1] += 1
        else:
            post.append(top[0])
            stack.pop()
    newid = {b: i for i, b in enumerate(post)}
    blocks, child_index, s0 = [], [], 0
    for b in post:
        length = len(tb[b][1])
        blocks.append(dict(seg=tb[b][0], length=length, s0=s0, parent=newid[bpar[b]] if bpar[b] >= 0 else -1,
                           n_child=len(bch[b]), child0=len(child_index)))
        child_index += [newid[c] for c in bch[b]]
        s0 += length
    return blocks, child_index, s0


class OraclePlan:
    """An nm_plan record for the oracle, built from input text."""

    def __init__(self, text: str):
        e, order = _entries(text)
        keep = []  # every array the record points into

        def arr(a, ctype):
            a = np.ascontiguousarray(a, dtype=np.float64 if ctype is C.c_double else np.int32)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(ctype))

        def get(cls, name, key, dflt=None):
            return e.get((cls, name, key), dflt)

        lats = order.get("lat", [])
        if len(lats) != 1:
            raise ValueError("exactly one lat")
        ln = lats[0]
        if int(get("lat", ln, "gradients", "1")) != 1:
            raise ValueError("the oracle's own builder takes 1-gradient lattices")
        P = PlanRecord()
        P.gradients = 1
        lt = get("lat", ln, "lattice_type")
        P.lattice_type, P.lambda_ = {"simple_cubic": (0, 1.0 / 6.0), "hexagonal": (1, 1.0 / 4.0)}[lt]
        P.geometry = {"planar": 0, "flat": 0, "cylindrical": 1, "spherical": 2}[get("lat", ln, "geometry", "planar")]
        P.stencil_full = 1
        MX = int(get("lat", ln, "n_layers"))
        P.MX, P.MY, P.MZ, P.JX, P.JY, P.M = MX, 0, 0, 1, 0, MX + 2
        M = P.M
        bcs = {"mirror": MIRROR, "periodic": PERIODIC, "surface": SURFACE}
        P.bc[0] = bcs[get("lat", ln, "lowerbound", "mirror")]
        P.bc[3] = bcs[get("lat", ln, "upperbound", "mirror")]
        off = float(get("lat", ln, "offset_first_layer", "0")) if P.geometry else 0.0
        P.offset_first_layer = max(off, 0.0)
        P.bond_length = float(get("lat", ln, "bondlength", "0"))
        L = np.zeros(M)
        if P.geometry == 0:
            L[1:MX + 1] = 1.0
            P.volume = MX
        else:
            lm1, l0, lp1 = np.zeros(M), np.zeros(M), np.zeros(M)
            lam = P.lambda_
            for x in range(1, MX + 1):
                r = P.offset_first_layer + 1.0 * x
                if P.geometry == 1:   # LGrad1::ComputeLambdas, cylinder
                    L[x] = PIE * (r ** 2 - (r - 1) ** 2)
                    lp1[x] = 2.0 * PIE * r / L[x] * lam
                    lm1[x] = 2.0 * PIE * (r - 1) / L[x] * lam
                    l0[x] = 1.0 - 2.0 * lam
                else:                 # sphere
                    L[x] = 4.0 / 3.0 * PIE * (r ** 3 - (r - 1) ** 3)
                    lp1[x] = 4.0 * PIE * r ** 2 / L[x] * lam
                    lm1[x] = 4.0 * PIE * (r - 1) ** 2 / L[x] * lam
                    l0[x] = 1.0 - lp1[x] - lm1[x]
            P.lambda_1, P.lambda0, P.lambda1 = arr(lm1, C.c_double), arr(l0, C.c_double), arr(lp1, C.c_double)
            o = P.offset_first_layer
            P.volume = (4.0 / 3.0 * PIE * ((MX + o) ** 3 - o ** 3) if P.geometry == 2
                        else PIE * ((MX + o) ** 2 - o ** 2))
        P.L = arr(L, C.c_double)
        # segments (mon), in order of first appearance
        segs = order.get("mon", [])
        ns = len(segs)
        segidx = {s: i for i, s in enumerate(segs)}
        freedom = np.zeros(ns, dtype=np.int32)
        mask = np.zeros((ns, M))

        def layer(tok, frozen, lo_bc, hi_bc):
            tok = tok.strip()
            if tok == "firstlayer":
                return 1
            if tok == "lastlayer":
                return MX
            if tok in ("lowerbound", "upperbound"):
                if not frozen or (lo_bc if tok == "lowerbound" else hi_bc) != SURFACE:
                    raise ValueError("a bound in a range needs a frozen segment and a surface")
                return 0 if tok == "lowerbound" else MX + 1
            return int(tok)

        for i, s in enumerate(segs):
            fr = get("mon", s, "freedom", "free")
            freedom[i] = {"free": SEG_FREE, "pinned": SEG_PINNED, "frozen": SEG_FROZEN}[fr]
            if get("mon", s, "valence") not in (None, "0"):
                raise ValueError("charged segments are outside the oracle's own builder")
            if freedom[i] != SEG_FREE:
                rng = get("mon", s, "pinned_range" if freedom[i] == SEG_PINNED else "frozen_range")
                rng = rng.replace("_x", "")
                lo, hi = (rng.split(";") + [None])[:2] if ";" in rng else (rng, rng)
                a = layer(lo, freedom[i] == SEG_FROZEN, P.bc[0], P.bc[3])
                b = layer(hi, freedom[i] == SEG_FROZEN, P.bc[0], P.bc[3])
                mask[i, a:b + 1] = 1.0
        chi = np.full((ns, ns), 123.0)
        for i, s in enumerate(segs):
            for k, t in enumerate(segs):
                v = get("mon", s, "chi_" + t)
                if v is not None:
                    chi[i, k] = float(v)
        chi = np.where(chi == 123.0, chi.T, chi)
        chi = np.where(chi == 123.0, 0.0, chi)
        if (np.diag(chi) != 0).any() or (chi != chi.T).any():
            raise ValueError("chi must be symmetric with a zero diagonal")
        ksam = np.ones(M, dtype=np.int32)
        for i in range(ns):
            if freedom[i] == SEG_FROZEN:
                ksam[mask[i] != 0] = 0
        gmask = np.where(freedom[:, None] == SEG_PINNED, mask * ksam, np.broadcast_to(ksam, (ns, M)))
        phi_frozen = np.where(freedom[:, None] == SEG_FROZEN, mask, 0.0)
        # molecules
        mols = order.get("mol", [])
        recs = (Molecule * len(mols))()
        keep.append(recs)
        P.solvent = P.neutralizer = -1
        molmons = []
        for m, mn in enumerate(mols):
            R = recs[m]
            if get("mol", mn, "Markov", "1") != "1":
                raise ValueError("Markov 2 chains are outside this builder's scope")
            comp = get("mol", mn, "composition")
            if comp.startswith("@"):
                raise ValueError("keyword compositions are outside the oracle's own builder")
            R.freedom = {"free": MOL_FREE, "restricted": MOL_RESTRICTED, "solvent": MOL_SOLVENT}[get("mol", mn, "freedom")]
            if R.freedom == MOL_SOLVENT:
                P.solvent = m
            if R.freedom == MOL_FREE:
                R.phibulk = float(get("mol", mn, "phibulk"))
            nodes, written = _composition(comp, segidx)
            branched = "[" in comp
            blocks, child_index, n_store = _blocks(nodes, written[0] if branched else written[-1])
            seq = [nodes[w][0] for w in written]
            if branched:
                seq = seq[::-1]
            mm = []
            for sg in seq:
                if sg not in mm:
                    mm.append(sg)
            N = float(sum(b["length"] for b in blocks))
            frac = np.zeros(len(mm))
            bl = (Block * len(blocks))()
            keep.append(bl)
            for j, b in enumerate(blocks):
                k = mm.index(b["seg"])
                frac[k] += b["length"]
                bl[j] = Block(b["seg"], k, b["length"], b["s0"], b["parent"], 1, 1.0, b["n_child"], b["child0"])
                if freedom[b["seg"]] == SEG_PINNED:
                    R.pinned = 1
            R.chainlength = N
            R.n_molmon = len(mm)
            R.molmon_seg = arr(mm, C.c_int)
            R.molmon_fraction = arr(frac / N, C.c_double)
            R.n_blocks = len(blocks)
            R.blocks = bl
            R.child_index = arr(child_index or [0], C.c_int)
            R.n_store = n_store
            R.markov = 1  # Markov 2 chains are outside this builder's scope (the key is refused)
            if R.freedom == MOL_RESTRICTED:
                if get("mol", mn, "n") is not None:
                    R.n = float(get("mol", mn, "n"))
                    R.theta = R.n * N
                else:
                    R.theta = float(get("mol", mn, "theta"))
                    R.n = R.theta / N
            molmons.append(mm)
        # iteration species: one per distinct χ row, in order of first
        # appearance over the molecules' monomer lists (system.cpp:430-500)
        seg_it = np.full(ns, -1, dtype=np.int32)
        it_seg, seen = [], []
        for mm in molmons:
            for sg in mm:
                if sg in seen:
                    continue
                seen.append(sg)
                same = [j for j, r in enumerate(it_seg) if (chi[sg] == chi[r]).all()]
                if same:
                    seg_it[sg] = same[0]
                else:
                    seg_it[sg] = len(it_seg)
                    it_seg.append(sg)
        P.n_seg = ns
        P.n_sp = ns
        P.scan_state = -1
        P.scan_reaction = -1
        names = (C.c_char_p * ns)(*[s.encode() for s in segs])
        mnames = (C.c_char_p * len(mols))(*[s.encode() for s in mols])
        keep += [names, mnames]
        P.seg_name, P.mol_name = names, mnames
        P.seg_freedom = arr(freedom, C.c_int)
        P.seg_it = arr(seg_it, C.c_int)
        P.seg_gmask = arr(gmask, C.c_double)
        P.seg_phi_frozen = arr(phi_frozen, C.c_double)
        P.chi = arr(chi, C.c_double)
        P.seg_valence = arr(np.zeros(ns), C.c_double)
        P.seg_epsilon = arr(np.full(ns, 80.0), C.c_double)
        P.ksam = arr(ksam, C.c_int)
        P.n_it = len(it_seg)
        P.it_seg = arr(it_seg, C.c_int)
        P.iv = P.n_it * M
        P.charged = 0
        P.n_mol = len(mols)
        P.mols = recs
        # newton (solve_scf.cpp:153-236 defaults)
        P.diis_m, P.iterationlimit, P.tolerance, P.deltamax, P.max_norm = 10, 1000, 1e-7, 0.1, 0
        for nn in order.get("newton", [])[:1]:
            P.tolerance = float(get("newton", nn, "tolerance", P.tolerance))
            P.deltamax = float(get("newton", nn, "deltamax", P.deltamax))
            P.diis_m = int(get("newton", nn, "m", P.diis_m))
            P.iterationlimit = int(get("newton", nn, "iterationlimit", P.iterationlimit))
            P.max_norm = int(get("newton", nn, "stop_criterion", "") == "max_of_element_of_|g|")
        if not 1 <= P.diis_m <= 100:
            P.diis_m = 10
        P.super_tolerance = 10.0 * P.tolerance
        P.super_iterationlimit = P.iterationlimit // 10
        P.super_deltamax = 0.5
        P.search_mol = P.search_what = P.target_kind = P.target_mol = P.target_what = -1
        P.scan_mol = P.scan_what = -1
        self.rec = P
        self._keep = keep
        self.M, self.iv, self.n_seg, self.n_mol = M, P.iv, ns, len(mols)

    @property
    def ptr(self) -> int:
        return C.addressof(self.rec)
