"""Oracle restatement of the libpll model arithmetic NetRAX relies on.

Test infrastructure only. libpll is not vendored in the reference (empty
``libs/raxml-ng`` submodule), so these follow the published methods:

* GTR / general time-reversible rate matrix, normalised to one expected
  substitution per unit time; eigensystem through the symmetric matrix
  ``Pi^1/2 Q Pi^-1/2``.
* ``P(t r) = U diag(exp(lambda r t)) U^-1``; a zero branch length gives the
  identity (the fake P-matrix of ``src/RaxmlWrapper.cpp:517-520``).
* Yang (1994) discrete Gamma with mean rates per category and equal weights
  (``PLL_GAMMA_RATES_MEAN``, ``src/RaxmlWrapper.cpp:621``).
* Nucleotide IUPAC tip encoding (A=1, C=2, G=4, T=8; gaps, N, ? = 15) and
  pattern compression with weights (``src/RaxmlWrapper.cpp:330``).
* Invariant sites for +I: a pattern is invariant in state j when the state
  masks of all its tips have exactly state j in common (their AND has one
  bit); the model's site likelihood is (1 - pinv) times the Gamma mixture
  (rates divided by 1 - pinv, so the mean rate stays 1) plus pinv times the
  frequency of that state (libpll's ``prop_invar``, set by NetRAX through
  raxml-ng's model, ``src/RaxmlWrapper.cpp:621-640``).
"""
import numpy as np
from scipy import special

DNA_CODES = {
    "A": 1, "C": 2, "G": 4, "T": 8, "U": 8,
    "M": 3, "R": 5, "W": 9, "S": 6, "Y": 10, "K": 12,
    "V": 7, "H": 11, "D": 13, "B": 14,
    "N": 15, "-": 15, "?": 15, "O": 15, "X": 15, ".": 15,
}


def rate_matrix(exch, freqs):
    """Normalised Q from upper-triangle exchangeabilities (row-major order)."""
    freqs = np.asarray(freqs, dtype=np.float64)
    S = freqs.size
    R = np.zeros((S, S))
    k = 0
    for i in range(S):
        for j in range(i + 1, S):
            R[i, j] = R[j, i] = exch[k]
            k += 1
    Q = R * freqs[None, :]
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    mu = -np.dot(freqs, np.diag(Q))
    return Q / mu


def eigensystem(exch, freqs):
    freqs = np.asarray(freqs, dtype=np.float64)
    Q = rate_matrix(exch, freqs)
    sq = np.sqrt(freqs)
    B = (sq[:, None] * Q) / sq[None, :]
    B = 0.5 * (B + B.T)
    lam, V = np.linalg.eigh(B)
    U = V / sq[:, None]
    Uinv = V.T * sq[None, :]
    return lam, U, Uinv, Q


def pmatrix(lam, U, Uinv, t):
    if t == 0.0:
        return np.eye(U.shape[0])
    return (U * np.exp(lam * t)[None, :]) @ Uinv


def pmatrices(lam, U, Uinv, t, rates):
    """[R][S][S] P-matrices for one branch length."""
    return np.ascontiguousarray(np.stack([pmatrix(lam, U, Uinv, t * r) for r in rates]))


def dpmatrices(lam, U, Uinv, t, rates):
    """d/dt of ``pmatrices``."""
    out = []
    for r in rates:
        out.append((U * (lam * r * np.exp(lam * r * t))[None, :]) @ Uinv)
    return np.ascontiguousarray(np.stack(out))


def gamma_rates_mean(alpha, ncat):
    """Yang (1994) mean rates of ``ncat`` equal-probability Gamma categories."""
    if ncat == 1:
        return np.ones(1)
    k = np.arange(1, ncat)
    cuts = special.gammaincinv(alpha, k / ncat) / alpha
    cdf1 = np.concatenate([[0.0], special.gammainc(alpha + 1.0, cuts * alpha), [1.0]])
    return ncat * np.diff(cdf1)


def encode_dna(seq):
    return np.array([DNA_CODES[c.upper()] for c in seq], dtype=np.uint32)


def compress_patterns(codes):
    """codes: [n_tips][n_sites] -> (unique [n_tips][n_pat], weights [n_pat])."""
    codes = np.asarray(codes)
    cols, inv, cnt = np.unique(codes.T, axis=0, return_inverse=True, return_counts=True)
    return np.ascontiguousarray(cols.T), cnt.astype(np.float64)


def tip_clv(codes, R, S):
    """Indicator CLV [n][R][S] for state-bitmask codes [n]."""
    bits = ((codes[:, None] >> np.arange(S)[None, :]) & 1).astype(np.float64)
    return np.ascontiguousarray(np.repeat(bits[:, None, :], R, axis=1))


def read_fasta(text):
    names, seqs, cur = [], [], None
    for line in text.splitlines():
        line = line.strip()
        if not line:
            continue
        if line.startswith(">"):
            names.append(line[1:].strip())
            seqs.append([])
            cur = seqs[-1]
        else:
            cur.append(line)
    return names, ["".join(s) for s in seqs]


def invariant_states(tip_codes):
    """Per pattern: the one state every tip admits, or -1 (libpll's
    invariant-site rule as described in the module docstring)."""
    codes = np.asarray(tip_codes, dtype=np.uint64)
    common = np.bitwise_and.reduce(codes, axis=0)
    single = (common != 0) & ((common & (common - np.uint64(1))) == 0)
    state = np.full(codes.shape[1], -1, dtype=np.int64)
    idx = np.nonzero(single)[0]
    if idx.size:
        state[idx] = np.log2(common[idx].astype(np.float64)).round().astype(np.int64)
    return state
