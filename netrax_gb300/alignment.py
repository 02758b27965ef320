"""Alignment front end: FASTA / PHYLIP text -> per-tip state masks in the
network's tip order -> pattern-compressed partitions for NetworkLikelihood.

Encoding and compression run in the library (``netlk_encode_states``,
``netlk_compress_patterns``); this module parses the text and orders the rows
by the network's tip labels.
"""
import ctypes

import numpy as np

from . import _native as N
from .synth import PartitionData


def read_fasta(text):
    """(names, sequences) of a FASTA text; sequence lines are concatenated."""
    names, seqs = [], []
    for line in text.splitlines():
        line = line.strip()
        if not line or line.startswith(";"):
            continue
        if line.startswith(">"):
            names.append(line[1:].strip().split()[0] if line[1:].strip() else "")
            seqs.append([])
        elif seqs:
            seqs[-1].append("".join(line.split()))
        else:
            raise ValueError("FASTA: sequence before the first header")
    return names, ["".join(s) for s in seqs]


def read_phylip(text):
    """(names, sequences) of a relaxed PHYLIP text, sequential or interleaved
    (first line: taxa and sites; names end at the first whitespace)."""
    lines = [ln for ln in text.splitlines() if ln.strip()]
    n, m = (int(x) for x in lines[0].split()[:2])
    names, seqs = [], []
    for ln in lines[1:1 + n]:
        parts = ln.split()
        names.append(parts[0])
        seqs.append("".join(parts[1:]))
    k = 0
    for ln in lines[1 + n:]:  # interleaved blocks: rows cycle through the taxa
        seqs[k % n] += "".join(ln.split())
        k += 1
    for nm, sq in zip(names, seqs):
        if len(sq) != m:
            raise ValueError("PHYLIP: %s has %d sites, header says %d" % (nm, len(sq), m))
    return names, seqs


def encode(seq, states=4):
    """State masks (uint32) of one sequence."""
    raw = seq.encode("ascii")
    out = np.zeros(len(raw), np.uint32)
    bad = ctypes.c_int64(-1)
    N.check(N.lib().netlk_encode_states(raw, len(raw), int(states),
                                         out.ctypes.data_as(N.c_uint32_p), ctypes.byref(bad)))
    return out


def compress(codes):
    """Distinct columns of codes [n_tips][n_sites] in first-occurrence order,
    and their multiplicities."""
    codes = np.ascontiguousarray(codes, np.uint32)
    n_tips, n_sites = codes.shape
    pat = np.zeros(n_tips * max(1, n_sites), np.uint32)
    w = np.zeros(max(1, n_sites))
    npat = ctypes.c_int64()
    N.check(N.lib().netlk_compress_patterns(codes.ctypes.data_as(N.c_uint32_p), n_tips, n_sites,
                                             pat.ctypes.data_as(N.c_uint32_p),
                                             w.ctypes.data_as(N.c_double_p), ctypes.byref(npat)))
    k = npat.value
    return np.ascontiguousarray(pat[:n_tips * k].reshape(n_tips, k)), w[:k].copy()


def partition_from_alignment(network, names, seqs, states=4, freqs=None, exch=None, alpha=1.0,
                             sites=None):
    """PartitionData for the columns ``sites`` (a slice or index array; all by
    default) with rows in the network's tip order. freqs default to the
    empirical state frequencies (ambiguous characters spread evenly over
    their states), exchangeabilities to all ones."""
    row = {nm: i for i, nm in enumerate(names)}
    missing = [network.labels[t] for t in range(network.n_tips) if network.labels[t] not in row]
    if missing:
        raise ValueError("alignment has no row for tips %s" % missing)
    codes = np.stack([encode(seqs[row[network.labels[t]]], states) for t in range(network.n_tips)])
    if sites is not None:
        codes = codes[:, sites]
    pat, w = compress(codes)
    if freqs is None:
        bits = ((codes[..., None] >> np.arange(states)) & 1).astype(np.float64)
        f = (bits / bits.sum(axis=-1, keepdims=True)).sum(axis=(0, 1))
        freqs = f / f.sum()
    if exch is None:
        exch = np.ones(states * (states - 1) // 2)
    return PartitionData(pat, w, np.asarray(freqs, np.float64), np.asarray(exch, np.float64), float(alpha),
                         int(codes.shape[1]), states=states)
