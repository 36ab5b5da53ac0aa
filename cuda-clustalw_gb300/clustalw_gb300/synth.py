"""Seeded synthetic sequence families for the benchmark workloads.

No public benchmark suite is named for this stage; these generators stand in
for the reference's FASTA fixtures with the shapes of the measured workloads:

* protein families: a root drawn i.i.d. from the Robinson & Robinson (1991)
  amino-acid background frequencies (Proc. Natl. Acad. Sci. USA 88:8880-8884),
  evolved down a random binary (Yule) tree; every branch substitutes each site
  with probability U(0.05, 0.3) and starts an indel at each site with
  probability 0.005, indel lengths geometric with mean 3, lengths held within
  +-10% of the root length;
* DNA families: uniform ACGT root, substitution U(0.05, 0.4), indel 0.01 with
  geometric mean length 4.

A Yule tree with N leaves is about 2 ln N branches deep, so applying those
per-branch rates unchanged drives most pairs of a 1000-sequence family to
background identity (~6%). To keep the 20-95% pairwise identity range the
workloads are defined with, both rates of every branch are multiplied by
min(1, depth / mean leaf depth), depth = 3 (protein) or 1.5 (DNA): the rates are per unit branch length
and the tree is rescaled to a fixed expected depth.

Sequences come out as ClustalW residue codes (index in
"ABCDEFGHIKLMNOPQRSTUVWXYZ-", alignment/Sequence.cpp:63-83).
"""
import numpy as np

from .pairwise import AMINO_ACID_CODES

# Robinson & Robinson (1991) background frequencies, one-letter order below.
_RR_LETTERS = "ARNDCQEGHILKMFPSTWYV"
_RR_FREQ = np.array(
    [
        0.07805, 0.05129, 0.04487, 0.05364, 0.01925, 0.04264, 0.06295, 0.07377, 0.02199, 0.05142,
        0.09019, 0.05744, 0.02243, 0.03856, 0.05203, 0.07120, 0.05841, 0.01330, 0.03216, 0.06441,
    ]
)
PROTEIN_CODES = np.array([AMINO_ACID_CODES.index(c) for c in _RR_LETTERS], dtype=np.int8)
PROTEIN_PROBS = _RR_FREQ / _RR_FREQ.sum()
DNA_CODES = np.array([AMINO_ACID_CODES.index(c) for c in "ACGT"], dtype=np.int8)
DNA_PROBS = np.full(4, 0.25)

# depth: the expected root-to-leaf branch count the rates are scaled to.
PROTEIN_MODEL = dict(codes=PROTEIN_CODES, probs=PROTEIN_PROBS, sub=(0.05, 0.3), indel=0.005, indel_mean=3.0, depth=3.0)
DNA_MODEL = dict(codes=DNA_CODES, probs=DNA_PROBS, sub=(0.05, 0.4), indel=0.01, indel_mean=4.0, depth=1.5)


def _evolve(seq, rng, model, lo, hi, scale):
    codes, probs = model["codes"], model["probs"]
    p_sub = rng.uniform(*model["sub"]) * scale
    out = seq.copy()
    mask = rng.random(len(out)) < p_sub
    n_sub = int(mask.sum())
    if n_sub:
        out[mask] = rng.choice(codes, size=n_sub, p=probs)
    n_ev = rng.binomial(len(out), model["indel"] * scale)
    if n_ev:
        pieces = list(out)
        for _ in range(n_ev):
            k = int(rng.geometric(1.0 / model["indel_mean"]))
            pos = int(rng.integers(0, len(pieces) + 1))
            insert = rng.random() < 0.5
            if insert and len(pieces) + k > hi:
                insert = False
            if not insert and len(pieces) - k < lo:
                insert = len(pieces) + k <= hi
                if not insert:
                    continue
            if insert:
                pieces[pos:pos] = list(rng.choice(codes, size=k, p=probs))
            else:
                del pieces[pos : pos + k]
        out = np.array(pieces, dtype=np.int8)
    return out


def family(nseqs, root_len, seed, model=PROTEIN_MODEL):
    """One family of `nseqs` leaves evolved from a root of length `root_len`."""
    rng = np.random.default_rng(seed)
    lo = max(1, int(np.floor(root_len * 0.9)))
    hi = max(lo, int(np.ceil(root_len * 1.1)))
    root = rng.choice(model["codes"], size=root_len, p=model["probs"]).astype(np.int8)
    # Topology first (Yule process: a uniformly chosen leaf splits), then the
    # depth-based rate scale, then the sequences top-down in split order.
    splits = []
    depth = [0]
    for _ in range(max(0, nseqs - 1)):
        i = int(rng.integers(len(depth)))
        splits.append(i)
        d = depth[i] + 1
        depth[i] = d
        depth.append(d)
    scale = min(1.0, model["depth"] / max(1.0, float(np.mean(depth))))
    leaves = [root]
    for i in splits:
        parent = leaves[i]
        leaves[i] = _evolve(parent, rng, model, lo, hi, scale)
        leaves.append(_evolve(parent, rng, model, lo, hi, scale))
    perm = rng.permutation(len(leaves))
    return [leaves[k] for k in perm[:nseqs]]


def protein_family(nseqs, root_len, seed):
    return family(nseqs, root_len, seed, PROTEIN_MODEL)


def dna_family(nseqs, root_len, seed):
    return family(nseqs, root_len, seed, DNA_MODEL)


def uneven_protein(nfamilies=8, per_family=125, lo=30, hi=2000, seed=0):
    """Families with root lengths log-uniform in [lo, hi], concatenated."""
    rng = np.random.default_rng(seed)
    seqs = []
    for f in range(nfamilies):
        L = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        seqs += protein_family(per_family, L, seed * 1000 + f + 1)
    return seqs


def length_limit_set(max_len=65535, seed=65535):
    """Sequences at the length limit: a max_len-residue random protein, a
    300-residue and a 100-residue fragment of it (20 % of the sites
    substituted, then about 1 % deleted), a 16,384-residue prefix of it and a
    mutated copy of that prefix (a pair whose Myers-Miller stage recurses 14
    levels)."""
    rng = np.random.default_rng(seed)

    def rand(length):
        pick = rng.choice(len(PROTEIN_CODES), size=length, p=PROTEIN_PROBS)
        return PROTEIN_CODES[pick].astype(np.int8)

    def mutate(seq, rate):
        seq = seq.copy()
        hit = rng.random(len(seq)) < rate
        seq[hit] = rand(int(hit.sum()))
        return seq[rng.random(len(seq)) >= 0.01]

    full = rand(max_len)
    return [full, mutate(full[30000:30300], 0.2), full[:16384].copy(), mutate(full[:16384], 0.2),
            mutate(full[100:200], 0.2)]


# The benchmark workloads (sizes as the reference's headline measurements use them).
WORKLOADS = {
    "protein-100x97": lambda seed=0: protein_family(100, 97, seed),
    "protein-1000x1523": lambda seed=0: protein_family(1000, 1523, seed),
    "protein-uneven-8x125": lambda seed=0: uneven_protein(8, 125, 30, 2000, seed),
    "dna-2000x1000": lambda seed=0: dna_family(2000, 1000, seed),
}


def serve_jobs(njobs, seed=0, n_range=(10, 500), len_range=(50, 1500)):
    """Job stream of the served workload: (nseqs, root_len, seed) per job."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(njobs):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        L = int(rng.integers(len_range[0], len_range[1] + 1))
        jobs.append((n, L, seed * 100003 + j))
    return jobs


def to_fasta(seqs, prefix="s"):
    lines = []
    for i, s in enumerate(seqs):
        lines.append(f">{prefix}{i + 1}")
        text = "".join("-" if c >= 30 else AMINO_ACID_CODES[c] for c in s)
        for k in range(0, len(text), 60):
            lines.append(text[k : k + 60])
    return "\n".join(lines) + "\n"


def all_pairs(n):
    """(si, sj) for si < sj in the reference's loop order."""
    iu = np.triu_indices(n, 1)
    return np.stack([iu[0], iu[1]], axis=1).astype(np.int32)
