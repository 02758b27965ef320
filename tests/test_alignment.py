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


def test_front_end_fuzz():
    """netlk_encode_states on arbitrary bytes (DNA): either every character is
    a known code (case-insensitive) and the masks are the table's, or the call
    returns NETLK_ERR_INVALID_ARGUMENT with the index of the first unknown one;
    netlk_compress_patterns equals a first-occurrence unique of the columns."""
    import ctypes
    from netrax_gb300 import _native as N
    dna = {"A": 1, "C": 2, "G": 4, "T": 8, "U": 8, "R": 5, "Y": 10, "S": 6, "W": 9, "K": 12, "M": 3, "B": 14,
           "D": 13, "H": 11, "V": 7, "N": 15, "?": 15, "-": 15, ".": 15, "O": 15, "X": 15}
    L = N.lib()
    rng = np.random.default_rng(11)
    alphabet = list(b"ACGTUNRYSWKMBDHV-?.xacgtnZ!")
    for it in range(2000):
        n = int(rng.integers(0, 30))
        if it % 2:
            raw = bytes(rng.integers(0, 256, size=n).astype(np.uint8))
        else:
            raw = bytes(rng.choice(alphabet, size=n).astype(np.uint8))
        out = np.zeros(max(1, n), np.uint32)
        bad = ctypes.c_int64(-7)
        st = L.netlk_encode_states(raw, n, 4, out.ctypes.data_as(N.c_uint32_p), ctypes.byref(bad))
        want_bad = next((i for i, c in enumerate(raw) if c >= 128 or chr(c).upper() not in dna), -1)
        if want_bad >= 0:
            assert st == N.NETLK_ERR_INVALID_ARGUMENT and bad.value == want_bad
        else:
            assert st == 0 and [int(x) for x in out[:n]] == [dna[chr(c).upper()] for c in raw]
    for _ in range(300):
        nt, ns = int(rng.integers(1, 6)), int(rng.integers(0, 50))
        codes = rng.integers(1, 4, size=(nt, ns)).astype(np.uint32)
        pat = np.zeros(nt * max(1, ns), np.uint32)
        w = np.zeros(max(1, ns))
        k = ctypes.c_int64(-1)
        assert L.netlk_compress_patterns(codes.ctypes.data_as(N.c_uint32_p), nt, ns, pat.ctypes.data_as(N.c_uint32_p),
                                         w.ctypes.data_as(N.c_double_p), ctypes.byref(k)) == 0
        order, count = [], {}
        for j in range(ns):
            c = tuple(codes[:, j])
            if c not in count:
                order.append(c)
                count[c] = 0
            count[c] += 1
        got = pat[:nt * k.value].reshape(nt, k.value)
        assert [tuple(got[:, j]) for j in range(k.value)] == order
        assert list(w[:k.value]) == [float(count[c]) for c in order]
