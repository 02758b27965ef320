"""Alignment front end: character encoding, pattern compression, FASTA /
PHYLIP reading into partitions in the network's tip order."""
import numpy as np
import pytest

from conftest import golden_cases
from netrax_gb300 import _native
from netrax_gb300.alignment import compress, encode, partition_from_alignment, read_fasta, read_phylip
from netrax_gb300.network import parse_extended_newick


def test_encode_dna_and_protein():
    assert list(encode("ACGTUacgt", 4)) == [1, 2, 4, 8, 8, 1, 2, 4, 8]
    assert list(encode("RYSWKMBDHV", 4)) == [5, 10, 6, 9, 12, 3, 14, 13, 11, 7]
    assert all(x == 15 for x in encode("N?-.OX", 4))
    order = "ARNDCQEGHILKMFPSTWYV"
    assert list(encode(order, 20)) == [1 << i for i in range(20)]
    assert list(encode("BZJ", 20)) == [(1 << 2) | (1 << 3), (1 << 5) | (1 << 6), (1 << 9) | (1 << 10)]
    assert all(x == (1 << 20) - 1 for x in encode("X?-.*", 20))
    with pytest.raises(_native.NetlkError) as e:
        encode("ACGTZ", 4)
    assert e.value.status == _native.NETLK_ERR_INVALID_ARGUMENT


def test_compress_matches_unique_columns():
    rng = np.random.default_rng(0)
    codes = (1 << rng.integers(0, 4, size=(7, 500))).astype(np.uint32)
    codes[:, 100:150] = codes[:, :50]  # repeats
    pat, w = compress(codes)
    assert w.sum() == codes.shape[1]
    # first-occurrence order, and every column is a pattern with its multiplicity
    cols = [tuple(c) for c in codes.T]
    firsts = []
    for c in cols:
        if c not in firsts:
            firsts.append(c)
    assert [tuple(c) for c in pat.T] == firsts
    for c, cnt in zip(firsts, w):
        assert cols.count(c) == cnt


def _fasta_of(case, rng):
    """FASTA text whose compressed columns are the golden case's patterns."""
    part = case["partitions"][0]
    ts = np.array(part["tip_states"], np.uint32)
    w = np.array(part["weights"], np.int64)
    cols = np.repeat(np.arange(ts.shape[1]), w)
    rng.shuffle(cols)
    inv = {1: "A", 2: "C", 4: "G", 8: "T", 15: "-", 5: "R", 10: "Y", 6: "S", 9: "W", 12: "K", 3: "M",
           14: "B", 13: "D", 11: "H", 7: "V"}
    lines = []
    for t, lab in enumerate(case["labels"]):
        lines.append(">" + lab)
        lines.append("".join(inv[int(x)] for x in ts[t, cols]))
    return "\n".join(lines) + "\n", ts, w


@pytest.mark.parametrize("name", ["smallNetwork", "celineNetwork", "threeReticulations"])
def test_fasta_partition_has_the_golden_patterns(name):
    case = [c for c in golden_cases() if c["name"] == name][0]
    text, ts, w = _fasta_of(case, np.random.default_rng(1))
    net = parse_extended_newick(case["newick"])
    names, seqs = read_fasta(text)
    pd = partition_from_alignment(net, names, seqs, states=4)
    got = sorted(zip(map(tuple, pd.tip_states.T), pd.weights))
    want = sorted(zip(map(tuple, ts.T), w.astype(float)))
    assert got == want
    assert pd.n_sites == int(w.sum())
    assert abs(pd.freqs.sum() - 1.0) < 1e-12


def test_phylip_sequential_and_interleaved():
    seq = "3 10\nA ACGTACGTAC\nB ACGTACGTAA\nC ACGTACGTCC\n"
    inter = "3 10\nA ACGTA\nB ACGTA\nC ACGTA\n\nCGTAC\nCGTAA\nCGTCC\n"
    assert read_phylip(seq) == read_phylip(inter) == (["A", "B", "C"], ["ACGTACGTAC", "ACGTACGTAA", "ACGTACGTCC"])
    with pytest.raises(ValueError):
        read_phylip("2 5\nA ACG\nB ACGTA\n")


@pytest.mark.gpu
def test_fasta_logl_matches_golden():
    from netrax_gb300.likelihood import NetworkLikelihood
    case = [c for c in golden_cases() if c["name"] == "smallNetwork"][0]
    text, _, _ = _fasta_of(case, np.random.default_rng(2))
    net = parse_extended_newick(case["newick"])
    part = case["partitions"][0]
    names, seqs = read_fasta(text)
    pd = partition_from_alignment(net, names, seqs, states=4, freqs=part["freqs"], exch=part["exch"],
                                  alpha=part["alpha"])
    with NetworkLikelihood(net, [pd], precision="fp64") as lik:
        assert lik.loglikelihood() == pytest.approx(case["AVERAGE"]["logl"], rel=1e-9)
