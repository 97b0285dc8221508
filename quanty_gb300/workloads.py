"""Synthetic workloads with the shapes of the reference's benchmark configurations.

* ``atomic()``: the 16-orbital 2p + 3d ion (2p orbitals 0-5, 3d orbitals 6-15; even = spin
  down, odd = spin up) as the reference's NewOperator("U"/"CF"/"ldots") builds it, read from
  ``data/atomic_2p3d.json`` (3d F2=10.0, F4=6.2, 10Dq=1.1, zeta3d=0.08; HX adds zeta2p=11.5 and
  the 2p-3d F2=6.2, G1=4.6, G3=2.6; dipoles Tx, Ty, Tz).
* ``anderson_impurity()``: the large discretised-bath Anderson impurity -- 86 spin-orbitals
  (2p, 3d, 7 bath shells of 10), 3d F0 = Udd = 7.5 plus the atomic multiplet terms, 2p-3d F0 =
  Upd = 8.5, bath energies uniform on [-5, 5] eV from seed 0, hybridisations from a 7-point
  discretisation of a semicircle density of states of half-width 2 eV (sum of V_k^2 = 4 eV^2,
  each bath orbital coupled to the 3d orbital of the same index), and a weak random real
  symmetric one-body field (<= 0.01 eV, seed 1) on the 3d shell that lifts the point-group
  symmetry so the closure of one determinant is the whole sector; every term is real.  Its sector: 2p6, 44
  electrons, at most 2 holes (particles) per filled (empty) shell, at most 3 holes in all
  filled shells together and at most 2 particles in all empty shells together: 47,481,880
  determinants.
"""
import json
import math
import os

import numpy as np

from .api import CREATION, Operator

HERE = os.path.dirname(os.path.abspath(__file__))


def _load():
    with open(os.path.join(HERE, "data", "atomic_2p3d.json")) as f:
        return json.load(f)


def atomic():
    d = _load()
    return {k: Operator(16, [(t[0], complex(t[1], t[2])) for t in d[k]], name=k) for k in ("H", "HX", "Tx", "Ty", "Tz")}


def ligand_field():
    """The 26-orbital ligand-field ion (2p 0-5, 3d 6-15, ligand 16-25) as the reference builds it
    (data/ligand_field_26.json): H, HX, Tx, Ty, Tz and the ground-state restrictions."""
    with open(os.path.join(HERE, "data", "ligand_field_26.json")) as f:
        d = json.load(f)
    ops = {k: Operator(26, [(t[0], complex(t[1], t[2])) for t in d[k]], name=k) for k in ("H", "HX", "Tx", "Ty", "Tz")}
    return ops, [tuple(r) for r in d["restrictions"]]


def number_pair(i, j, value):
    """n_i n_j (i != j) in the normal order the reference stores two-body terms in:
    c^dag_a c^dag_b c_a c_b with a > b (ladder codes [b, a, b^dag, a^dag], the rightmost
    acting first) and value -U, since n_a n_b = -c^dag_a c^dag_b c_a c_b."""
    a, b = max(i, j), min(i, j)
    return [b, a, b | CREATION, a | CREATION], -value


def merged(terms):
    """Sum the values of identical ladder strings (the reference's operator addition)."""
    acc, order = {}, []
    for ops, v in terms:
        k = tuple(ops)
        if k not in acc:
            acc[k] = 0j
            order.append(k)
        acc[k] += v
    return [(list(k), acc[k]) for k in order if acc[k] != 0]


def anderson_impurity(nshell=7, seed=0, udd=7.5, upd=8.5, half_width=2.0, v2_total=4.0, hole_max=3,
                      particle_max=2, field=0.01, delta=0.0, core_holes=0, complex_field=False):
    """Returns (H, restrictions, seed determinant, info dict)."""
    nf = 16 + 10 * nshell
    at = _load()
    terms = [(list(t[0]), complex(t[1], t[2])) for t in at["HX"]]
    d_orb = list(range(6, 16))
    p_orb = list(range(0, 6))
    if delta:  # charge-transfer shift of the 3d level
        for d in d_orb:
            terms.append(([d, d | CREATION], float(delta)))
    for a in range(10):
        for b in range(a + 1, 10):
            terms.append(number_pair(d_orb[a], d_orb[b], udd))
    for p in p_orb:
        for d in d_orb:
            terms.append(number_pair(p, d, upd))
    rng = np.random.default_rng(seed)
    eps = np.sort(rng.uniform(-5.0, 5.0, nshell))
    x = -half_width + 2 * half_width * (np.arange(nshell) + 0.5) / nshell
    w = np.sqrt(1 - (x / half_width) ** 2)
    V = np.sqrt(v2_total * w / w.sum())
    for k in range(nshell):
        for a in range(10):
            b = 16 + 10 * k + a
            d = d_orb[a]
            terms.append(([b, b | CREATION], float(eps[k])))
            terms.append(([b, d | CREATION], float(V[k])))
            terms.append(([d, b | CREATION], float(V[k])))
    # a weak random one-body field on the 3d shell (seed + 1, entries up to `field` eV) breaks
    # the point-group symmetry, so the closure of the seed determinant under H is the whole
    # restricted sector rather than one symmetry block of it.  It is real symmetric, like the
    # rest of this Hamiltonian (the reference's atomic H and HX carry real values only);
    # complex_field=True draws a complex Hermitian one instead (same connectivity, so the
    # same sector), which makes every impurity move complex-valued.
    fr = np.random.default_rng(seed + 1)
    for a in range(10):
        for b in range(a, 10):
            re = fr.uniform(-1, 1)
            im = fr.uniform(-1, 1) if a != b else 0.0
            v = field * complex(re, im if complex_field else 0.0)
            terms.append(([d_orb[b], d_orb[a] | CREATION], v))
            if a != b:
                terms.append(([d_orb[a], d_orb[b] | CREATION], v.conjugate()))
    H = Operator(nf, merged(terms), name="AndersonImpurity")
    filled = [k for k in range(nshell) if eps[k] < 0]
    empty = [k for k in range(nshell) if eps[k] >= 0]

    def mask(orbs):
        s = ["0"] * nf
        for o in orbs:
            s[o] = "1"
        return "".join(s)

    R = [(mask(p_orb), 6 - core_holes, 6)]
    for k in filled:
        R.append((mask(range(16 + 10 * k, 26 + 10 * k)), 8, 10))
    for k in empty:
        R.append((mask(range(16 + 10 * k, 26 + 10 * k)), 0, 2))
    fo = [o for k in filled for o in range(16 + 10 * k, 26 + 10 * k)]
    eo = [o for k in empty for o in range(16 + 10 * k, 26 + 10 * k)]
    R.append((mask(fo), len(fo) - hole_max, len(fo)))
    R.append((mask(eo), 0, particle_max))
    seed_det = mask(p_orb + d_orb[:8] + fo)
    info = {"nf": nf, "bath_energies": eps.tolist(), "V": V.tolist(), "filled_shells": filled,
            "electrons": 6 + 8 + len(fo),
            "sector_determinants": sector_size(len(filled), len(empty), hole_max=hole_max, particle_max=particle_max)}
    return H, R, seed_det, info


def sector_size(nfilled, nempty, nd0=8, hole_max=3, particle_max=2, per_shell=2):
    """Number of determinants in the restricted sector (counted combinatorially)."""
    def dist(nsh, mx):
        poly = {0: 1}
        for _ in range(nsh):
            new = {}
            for t, c in poly.items():
                for h in range(per_shell + 1):
                    if t + h <= mx:
                        new[t + h] = new.get(t + h, 0) + c * math.comb(10, h)
            poly = new
        return poly
    H, P = dist(nfilled, hole_max), dist(nempty, particle_max)
    tot = 0
    for h, ch in H.items():
        for p, cp in P.items():
            nd = nd0 + h - p
            if 0 <= nd <= 10:
                tot += ch * cp * math.comb(10, nd)
    return tot


def _bits_to_bytes(rows, nf):
    bits = np.zeros((len(rows), ((nf + 7) // 8) * 8), dtype=np.uint8)
    for r, orbs in enumerate(rows):
        bits[r, list(orbs)] = 1
    return np.packbits(bits, axis=1, bitorder="big")


def anderson_sector_bytes(info, nf, hole_max=3, particle_max=2, per_shell=2):
    """All determinants of the anderson_impurity() sector in the reference byte layout,
    built on the host by products of shell configurations (no GPU involved)."""
    import itertools
    nsh = (nf - 16) // 10
    filled = list(info["filled_shells"])
    empty = [k for k in range(nsh) if k not in filled]
    fo = [o for k in filled for o in range(16 + 10 * k, 26 + 10 * k)]
    eo = [o for k in empty for o in range(16 + 10 * k, 26 + 10 * k)]

    def shell_of(o):
        return (o - 16) // 10

    def ok_per_shell(sel):
        cnt = {}
        for o in sel:
            cnt[shell_of(o)] = cnt.get(shell_of(o), 0) + 1
        return all(v <= per_shell for v in cnt.values())

    F = {}  # holes -> occupied filled-shell orbitals
    for h in range(hole_max + 1):
        F[h] = [tuple(o for o in fo if o not in hs) for hs in itertools.combinations(fo, h) if ok_per_shell(hs)]
    P = {}
    for p in range(particle_max + 1):
        P[p] = [ps for ps in itertools.combinations(eo, p) if ok_per_shell(ps)]
    Fb = {h: _bits_to_bytes(v, nf) for h, v in F.items()}
    Pb = {p: _bits_to_bytes(v, nf) for p, v in P.items()}
    core = _bits_to_bytes([range(0, 6)], nf)[0]
    out = []
    d_orb = list(range(6, 16))
    for h in F:
        for p in P:
            nd = 8 + h - p
            if not 0 <= nd <= 10:
                continue
            D = _bits_to_bytes(list(itertools.combinations(d_orb, nd)), nf) | core
            fp = (Fb[h][:, None, :] | Pb[p][None, :, :]).reshape(-1, Fb[h].shape[1])
            for drow in D:
                out.append(fp | drow)
    return np.concatenate(out)
