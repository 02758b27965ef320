"""Model helpers used on the host by the workload generator and the harness.

The library evaluates its own model math (``csrc/model.cpp``); these numpy /
scipy versions only drive sequence simulation and state encoding.
"""
import numpy as np
from scipy import special

# IUPAC nucleotide codes -> 4-bit state masks (A=1, C=2, G=4, T=8)
DNA_MASK = {
    "A": 1, "C": 2, "G": 4, "T": 8, "U": 8, "M": 3, "R": 5, "W": 9, "S": 6,
    "Y": 10, "K": 12, "V": 7, "H": 11, "D": 13, "B": 14,
    "N": 15, "-": 15, "?": 15, "O": 15, "X": 15, ".": 15,
}


def rate_matrix(freqs, exch):
    freqs = np.asarray(freqs, np.float64)
    S = freqs.size
    Q = np.zeros((S, S))
    iu = np.triu_indices(S, 1)
    Q[iu] = exch
    Q = Q + Q.T
    Q = Q * freqs[None, :]
    np.fill_diagonal(Q, -Q.sum(axis=1))
    return Q / -np.dot(freqs, np.diag(Q))


def eigen(freqs, exch):
    freqs = np.asarray(freqs, np.float64)
    Q = rate_matrix(freqs, exch)
    sq = np.sqrt(freqs)
    B = sq[:, None] * Q / sq[None, :]
    lam, V = np.linalg.eigh(0.5 * (B + B.T))
    return lam, V / sq[:, None], V.T * sq[None, :]


def gamma_mean_rates(alpha, ncat):
    if ncat == 1:
        return np.ones(1)
    cuts = special.gammaincinv(alpha, np.arange(1, ncat) / ncat)
    cdf = np.concatenate([[0.0], special.gammainc(alpha + 1.0, cuts), [1.0]])
    return ncat * np.diff(cdf)


def encode_dna(seqs):
    """List of equal-length strings -> uint32 masks [n_seqs][n_sites]."""
    return np.array([[DNA_MASK[c.upper()] for c in s] for s in seqs], dtype=np.uint32)


def compress_patterns(codes):
    cols, counts = np.unique(np.asarray(codes).T, axis=0, return_counts=True)
    return np.ascontiguousarray(cols.T.astype(np.uint32)), counts.astype(np.float64)
