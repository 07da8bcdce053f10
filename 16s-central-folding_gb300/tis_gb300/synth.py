"""Seeded synthetic TIS RNA systems written in the reference's input formats.

The reference reads four files (src/16SCD_Mg_Cl_K_COPY_fast.cpp, main() at 6038):
  * a PDB whose heavy atoms are averaged into P / S / B beads (read_PDB, 3137),
  * an "unprocessed bonds" file of hydrogen-bond candidates (3733),
  * an "unprocessed stacks" file of tertiary stacks (4232),
  * the 9-type parameter table MAXIKEY (read_maxi_key, 2883).
This module writes all four for a generated chain, so the reference engine, the
CPU oracle and the GPU path all load the same system through the same parser.

Conventions the reference's parser imposes (and this generator honours):
  * the chain starts with a nucleotide without a 5' phosphate, so the bead
    order is S1 B1 P2 S2 B2 ... and n_nt nucleotides give 3 n_nt - 1 beads;
  * one heavy atom per bead (P, O5', N9 for purines / N1 for pyrimidines), so
    the bead centroid is that atom;
  * residue numbers 562..841 then 848.. (the reference maps RES<842 to RES-561
    and the rest to RES-567, lines 3783-3795 and 4290-4300);
  * tokens are separated by spaces (the reader splits on white space and takes
    tokens 3/4/7/8/9 as atom name, residue name, x, y, z).
"""
import os

import numpy as np

# MAXIKEY_Mg_Cl_K.dat: type, mass (amu), LJ radius (A), LJ depth (kcal/mol), charge.
# Types 1-6 are P, S, B(A), B(G), B(C), B(U); 7 Mg2+, 8 Cl-, 9 K+.
MAXIKEY_TABLE = [
    (1, 62.9740, 2.1000, 0.200000, -1),
    (2, 131.106, 2.9000, 0.200000, 0),
    (3, 134.132, 2.8000, 0.200000, 0),
    (4, 150.132, 3.0000, 0.200000, 0),
    (5, 110.102, 2.7000, 0.200000, 0),
    (6, 111.084, 2.7000, 0.200000, 0),
    (7, 24.3050, 0.7926, 0.894700, 2),
    (8, 35.4500, 1.9480, 0.265000, -1),
    (9, 39.1000, 2.6580, 0.000328, 1),
]

# Equilibrium bonded geometry of the force field (polymer_constraints, 2354-2520):
# S-B bond and the B-S-P angles per base, S(i)-P(i+1), P(i)-S(i), and the two
# backbone angles.  Used only to grow a strain-free starting chain.
_R_SB = {"A": 4.8515, "C": 4.2738, "G": 4.9659, "U": 4.2733}
_ALPHA1 = {"A": 1.9259, "C": 1.9655, "G": 1.9150, "U": 1.9663}
_ALPHA2 = {"A": 1.7029, "C": 1.5803, "G": 1.7690, "U": 1.5735}
_R_SP = 3.8157   # S(i) - P(i+1)
_R_PS = 4.6010   # P(i) - S(i)
_BETA1 = 1.5256  # S(i) - P(i) - S(i-1)
_BETA2 = 1.4440  # P(i+1) - S(i) - P(i)

_BASE_ATOM = {"A": "N9", "G": "N9", "C": "N1", "U": "N1"}
# Watson-Crick / wobble atom pairs written as CAN11 lines (names understood by
# return_HB_JNDX, 3636-3667).
_PAIR_ATOMS = {
    ("A", "U"): ["N6", "O4", "N1", "N3"],
    ("U", "A"): ["O4", "N6", "N3", "N1"],
    ("G", "C"): ["O6", "N4", "N1", "N3", "N2", "O2"],
    ("C", "G"): ["N4", "O6", "N3", "N1", "O2", "N2"],
    ("G", "U"): ["O6", "N3", "N1", "O2"],
    ("U", "G"): ["N3", "O6", "O2", "N1"],
}


def resnum(t):
    """PDB residue number of nucleotide t (1-based) in the reference's numbering."""
    return 561 + t if t <= 280 else 567 + t


def _unit(v):
    return v / np.linalg.norm(v)


def _direction(rng, prev_bond, theta, jitter):
    """Random unit vector d with angle(-prev_bond, d) close to theta."""
    a = _unit(-prev_bond)
    tmp = rng.normal(size=3)
    p = _unit(tmp - tmp.dot(a) * a)
    # a x p, as numpy.cross forms it (products, then one subtraction per component)
    q = np.array([a[1] * p[2] - a[2] * p[1], a[2] * p[0] - a[0] * p[2], a[0] * p[1] - a[1] * p[0]])
    th = theta + rng.normal() * jitter
    phi = rng.uniform(0, 2 * np.pi)
    return np.cos(th) * a + np.sin(th) * (np.cos(phi) * p + np.sin(phi) * q)


def grow_chain(seq, rng, r_conf, min_sep=3.6, tries=400):
    """Confined self-avoiding walk of the TIS chain; returns bead positions in
    PDB order (S1 B1 P2 S2 B2 ...) and, per nucleotide, its (P, S, B) bead ids."""
    n = len(seq)
    pos = []
    ids = []
    buf = np.empty((3 * n, 3))  # pos as one array (rows [0, len(pos)))

    def ok(p, exclude):
        if np.linalg.norm(p) > r_conf:
            return False
        if not pos:
            return True
        arr = buf[:len(pos)]
        d2 = ((arr - p) ** 2).sum(1)
        if exclude:
            d2[list(exclude)] = 1e9
        return d2.min() >= min_sep * min_sep

    def place(origin, r0, prev_bond, theta, exclude):
        for attempt in range(tries):
            jitter = 0.15 if attempt < tries // 2 else 0.6
            if prev_bond is None:
                d = _unit(rng.normal(size=3))
            else:
                d = _direction(rng, prev_bond, theta, jitter)
            p = origin + r0 * d
            if ok(p, exclude):
                return p
        # crowded: give up the confinement but keep excluded volume if possible
        for _ in range(tries):
            p = origin + r0 * _unit(rng.normal(size=3))
            arr = buf[:len(pos)]
            d2 = ((arr - p) ** 2).sum(1)
            if exclude:
                d2[list(exclude)] = 1e9
            if d2.min() >= min_sep * min_sep:
                return p
        return origin + r0 * _unit(rng.normal(size=3))

    def add(p):
        buf[len(pos)] = p
        pos.append(p)

    s_prev = p_prev = None
    for t in range(n):
        b = seq[t]
        if t == 0:
            s = np.zeros(3)
            add(s)
            sid = 0
            bpos = place(s, _R_SB[b], None, 0.0, {sid})
            add(bpos)
            ids.append((-1, sid, sid + 1))
            s_prev, p_prev = s, None
            continue
        sid_prev = ids[-1][1]
        prev_bond = (s_prev - p_prev) if p_prev is not None else (s_prev - pos[ids[-1][2]])
        theta = _BETA2 if p_prev is not None else _ALPHA1[seq[t - 1]]
        # only the bonded origin is exempt from the overlap test: 1-3 partners must
        # also stay apart, or the bond angle collapses onto its neighbour
        p = place(s_prev, _R_SP, prev_bond, theta, {sid_prev})
        pid = len(pos)
        add(p)
        s = place(p, _R_PS, p - s_prev, _BETA1, {pid})
        sid = len(pos)
        add(s)
        bpos = place(s, _R_SB[b], s - p, _ALPHA2[b], {sid})
        add(bpos)
        ids.append((pid, sid, sid + 1))
        s_prev, p_prev = s, p
    return np.asarray(pos), ids


def _pick_close_pairs(rng, B, ok_pair, n_want, pool_factor=3, max_dist=12.0):
    n = len(B)
    d = np.sqrt(((B[:, None, :] - B[None, :, :]) ** 2).sum(-1))
    cand = [(d[i, j], i, j) for i in range(n) for j in range(i + 1, n) if ok_pair(i, j) and d[i, j] < max_dist]
    cand.sort()
    pool = cand[: max(n_want * pool_factor, n_want)]
    if len(pool) < n_want:  # not enough close pairs: top up with random admissible ones
        extra = [(d[i, j], i, j) for i in range(n) for j in range(i + 1, n) if ok_pair(i, j) and d[i, j] >= max_dist]
        rng.shuffle(extra)
        pool += extra[: n_want - len(pool)]
    sel = rng.choice(len(pool), size=min(n_want, len(pool)), replace=False)
    return [pool[k][1:] for k in sorted(sel)]


def generate(out_dir, name, n_nt, seed, n_hb_pairs, n_tertiary=None, density=400.0):
    """Writes <name>.pdb, <name>_bonds.dat, <name>_stacks.dat and MAXIKEY_Mg_Cl_K.dat
    into out_dir; returns a dict of the four paths plus the sequence."""
    rng = np.random.default_rng(seed)
    seq = "".join(rng.choice(list("ACGU"), size=n_nt))
    n_beads = 3 * n_nt - 1
    r_conf = (3.0 * n_beads * density / (4.0 * np.pi)) ** (1.0 / 3.0)
    pos, ids = grow_chain(seq, rng, r_conf)
    pos = pos - pos.min(0) + 10.0
    os.makedirs(out_dir, exist_ok=True)

    pdb = os.path.join(out_dir, f"{name}.pdb")
    serial = 1
    with open(pdb, "w") as f:
        for t in range(n_nt):
            p_id, s_id, b_id = ids[t]
            rn = resnum(t + 1)
            atoms = []
            if p_id >= 0:
                atoms.append(("P", p_id, "P"))
            atoms.append(("O5'", s_id, "O"))
            atoms.append((_BASE_ATOM[seq[t]], b_id, "N"))
            for an, bid, el in atoms:
                x, y, z = pos[bid]
                f.write(f"ATOM {serial:6d} {an:<4s} {seq[t]:>3s} A {rn:5d}    {x:.3f} {y:.3f} {z:.3f}  1.00  0.00 {el}\n")
                serial += 1

    B = np.asarray([pos[ids[t][2]] for t in range(n_nt)])
    comp = set(_PAIR_ATOMS.keys())

    def hb_ok(i, j):  # 0-based nucleotides; both need a following P (index <= n-2)
        return j - i >= 4 and i <= n_nt - 2 and j <= n_nt - 2 and (seq[i], seq[j]) in comp

    bonds = os.path.join(out_dir, f"{name}_bonds.dat")
    pairs = _pick_close_pairs(rng, B, hb_ok, n_hb_pairs) if n_hb_pairs > 0 else []
    lines = [f"CAN11 {resnum(i + 1)} {resnum(j + 1)} {' '.join(_PAIR_ATOMS[(seq[i], seq[j])])} TER" for i, j in pairs]
    if not lines:
        raise ValueError("the reference's bonds reader needs at least one record")
    with open(bonds, "w") as f:  # no newline after the last TER: the reference's reader loops on feof()
        f.write("\n".join(lines))

    if n_tertiary is None:
        n_tertiary = max(1, n_nt // 8)

    def st_ok(i, j):  # '-' site needs the preceding P, i.e. nucleotide index >= 1
        return j - i >= 3 and 1 <= i and j <= n_nt - 2

    stacks = os.path.join(out_dir, f"{name}_stacks.dat")
    st_pairs = _pick_close_pairs(rng, B, st_ok, n_tertiary, max_dist=9.0)
    with open(stacks, "w") as f:
        for i, j in st_pairs:
            s1 = "+" if rng.uniform() < 0.5 else "-"
            s2 = "+" if rng.uniform() < 0.5 else "-"
            f.write(f"{s1}{resnum(i + 1)} {s2}{resnum(j + 1)}\n")

    maxikey = os.path.join(out_dir, "MAXIKEY_Mg_Cl_K.dat")
    write_maxikey(maxikey)
    return {"pdb": pdb, "bonds": bonds, "stacks": stacks, "maxikey": maxikey, "sequence": seq}


def write_maxikey(path):
    with open(path, "w") as f:
        for t, m, r, e, q in MAXIKEY_TABLE:
            f.write(f"{t} {m} {r:.4f} {e:.6f} {q}\n")


# Workloads named by what they are (sizes from the benchmark description):
#   small:   76-nt chain,  200 A box, 2 mM MgCl2 + 50 mM KCl (10 Mg, 317 K, 261 Cl)
#   central: 346-nt chain, 350 A box, 5 mM MgCl2 + 76 mM KCl (129 Mg, 2307 K, 2219 Cl)
#   large:   1500-nt chain, 600 A box, 10 mM MgCl2 + 150 mM KCl (1300 Mg, 21000 K, 22100 Cl)
WORKLOADS = {
    "small": dict(n_nt=76, box=200.0, n_hb_pairs=20, ions=(10, 261, 317), seed=1000),
    "central": dict(n_nt=346, box=350.0, n_hb_pairs=120, ions=(129, 2219, 2307), seed=2000),
    "large": dict(n_nt=1500, box=600.0, n_hb_pairs=400, ions=(1300, 22100, 21000), seed=4000),
}


def ion_counts_for(cmg_molar, ck_molar, box, n_entries):
    """Ion numbers by the reference's rule (E:6167-6171): Mg and K from the bulk
    concentrations, Cl neutralising the RNA's (n_entries-1)/2 phosphates."""
    vol = box ** 3
    n_mg = int(cmg_molar * 6.022 * 0.0001 * vol)
    n_k = int(ck_molar * 6.022 * 0.0001 * vol)
    n_cl = 2 * n_mg + n_k - (n_entries - 1) // 2
    return n_mg, n_cl, n_k


def batch_mg_sweep(n_replicas=64, mg_max_mm=20.0, kcl_mm=76.0, box=350.0, n_nt=346):
    """Per-replica (Mg, Cl, K) counts for an Mg2+ sweep 0..mg_max in n_replicas linear
    steps at fixed KCl: Mg and K from the reference's count rule, Cl neutralising."""
    n_entries = 2 * n_nt - 1
    out = []
    for r in range(n_replicas):
        cmg = (mg_max_mm * r / max(1, n_replicas - 1)) * 1e-3
        out.append(ion_counts_for(cmg, kcl_mm * 1e-3, box, n_entries))
    return out
