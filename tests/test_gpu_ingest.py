"""GPU FASTA ingest (blamm_fasta_parse_device) against the oracle's restatement of
FastaBatch: same stream bases, same run starts, sequence indices and positions."""
import os

import numpy as np
import pytest

from golden_cases import GOLDEN
from test_host_cpu import _oracle_stream

pytestmark = pytest.mark.gpu


def _gpu_parse(scanner, raw: bytes):
    torch = pytest.importorskip("torch")
    n = len(raw)
    d_raw = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
    d_b = torch.empty(max(n, 1), dtype=torch.uint8, device="cuda")
    d_rs, d_rq, d_rp, d_h = (torch.empty(max(n, 1), dtype=torch.int64, device="cuda") for _ in range(4))
    nucl = np.zeros(4, dtype=np.uint64)
    nb, nr, ns = scanner.fasta_parse_device(d_raw.data_ptr(), n, d_b.data_ptr(), d_rs.data_ptr(), d_rq.data_ptr(),
                                            d_rp.data_ptr(), d_h.data_ptr(), nucl)
    return (d_b[:nb].cpu().numpy(), d_rs[:nr].cpu().numpy(), d_rq[:nr].cpu().numpy(), d_rp[:nr].cpu().numpy(),
            d_h[:ns].cpu().numpy(), nucl)


def _concat(files):
    parts = []
    for f in files:
        b = open(f, "rb").read()
        parts.append(b if b.endswith(b"\n") else b + b"\n")
    return b"".join(parts)


def _check(scanner, files):
    raw = _concat(files)
    got = _gpu_parse(scanner, raw)
    want = _oracle_stream(files)
    for name, g, w in zip(("bases", "run_start", "run_seq", "run_seqpos"), got[:4], want):
        assert np.array_equal(g, w), f"{name}: {g[:8]} vs {w[:8]}"
    hp = got[4]
    assert all(raw[int(p)] == ord(">") for p in hp)
    # the dict module's nucleotide composition of the stream
    low = want[0] | 0x20
    assert [int(x) for x in got[5]] == [int(np.count_nonzero(low == ord(c))) for c in "acgt"]
    return got


def test_golden_fasta_files(scanner):
    files = [os.path.join(GOLDEN, "mixed", "seqs", f) for f in ("a_file.fa", "b_file.fa")]
    _check(scanner, files)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_fasta_with_n_runs_lowercase_crlf_and_empty_lines(scanner, tmp_path, seed):
    rng = np.random.default_rng(seed)
    files = []
    for fi in range(3):
        lines = []
        for si in range(int(rng.integers(1, 6))):
            lines.append(f">seq{fi}_{si} some description")
            L = int(rng.integers(0, 20_000))
            s = rng.choice(np.frombuffer(b"ACGTACGTacgtNNnRY", dtype=np.uint8), size=L)
            # N runs
            for _ in range(int(rng.integers(0, 4))):
                a = int(rng.integers(0, max(1, L)))
                s[a:a + int(rng.integers(1, 500))] = ord("N")
            w = int(rng.integers(1, 120))
            eol = "\r\n" if rng.random() < 0.3 else "\n"
            for k in range(0, L, w):
                lines.append(s[k:k + w].tobytes().decode() + ("" if eol == "\n" else "\r"))
                if rng.random() < 0.02:
                    lines.append("")
        p = tmp_path / f"f{fi}.fa"
        p.write_bytes(("\n".join(lines) + "\n").encode())
        files.append(str(p))
    _check(scanner, files)


def test_sequence_before_header_is_rejected(scanner):
    from blamm_gb300 import BlammError
    with pytest.raises(BlammError):
        _gpu_parse(scanner, b"ACGT\n>s\nACGT\n")


def test_nucleotide_counts_equal_the_reference_dictionary(scanner, tmp_path):
    """The two-sequence case's sequences.mf.dict (written by the reference's dict module) holds
    NUCL_COUNT_ACGT of its FASTA file (stored gzip-compressed); the GPU ingest gives the same
    four counts."""
    import gzip
    d = os.path.join(GOLDEN, "two_sequences_1mbp")
    words = open(os.path.join(d, "expected", "sequences.mf.dict")).read().split()
    want = [int(x) for x in words[words.index("NUCL_COUNT_ACGT") + 1:][:4]]
    fa = tmp_path / "seqs.fa"
    fa.write_bytes(gzip.open(os.path.join(d, "seqs", "seqs.fa.gz")).read())
    got = _gpu_parse(scanner, _concat([str(fa)]))
    assert [int(x) for x in got[5]] == want


def _random_fasta(tmp_path, seed: int, nfiles: int = 3, maxlen: int = 20_000):
    rng = np.random.default_rng(seed)
    files = []
    for fi in range(nfiles):
        lines = []
        for si in range(int(rng.integers(1, 6))):
            lines.append(f">seq{fi}_{si} description")
            L = int(rng.integers(0, maxlen))
            s = rng.choice(np.frombuffer(b"ACGTACGTacgtNNnRY", dtype=np.uint8), size=L)
            for _ in range(int(rng.integers(0, 4))):
                a = int(rng.integers(0, max(1, L)))
                s[a:a + int(rng.integers(1, 500))] = ord("N")
            w = int(rng.integers(1, 120))
            for k in range(0, L, w):
                lines.append(s[k:k + w].tobytes().decode())
        p = tmp_path / f"r{seed}_{fi}.fa"
        p.write_bytes(("\n".join(lines) + "\n").encode())
        files.append(str(p))
    return files


def _chunk_runs(run_start, begin, size):
    """The run starts inside [begin, begin + size), relative to begin, led by the run in
    effect at begin (FastaStream::nextChunk's markers)."""
    k = int(np.searchsorted(run_start, begin, side="right")) - 1
    inner = run_start[(run_start > begin) & (run_start < begin + size)] - begin
    return np.concatenate([[0], inner]).astype(np.int64) if k >= 0 else inner


@pytest.mark.parametrize("seed", [3, 4])
def test_resident_stream_equals_the_oracle_stream_and_scans_in_chunks(scanner, tmp_path, seed):
    """blamm_stream_load_fasta keeps FastaBatch's stream on the device: its run table equals the
    oracle's, and blamm_scan_stream over overlapping chunks of it gives the whole stream's hits."""
    import oracle
    from bankutil import make_bank, same_hits
    files = _random_fasta(tmp_path, seed)
    raw = _concat(files)
    nb, nr, ns, nucl = scanner.stream_load_fasta(raw)
    bases, run_start, run_seq, run_seqpos = _oracle_stream(files)
    rs, rq, rp, hp = scanner.stream_tables()
    assert nb == len(bases) and nr == len(run_start) and ns == raw.count(b"\n>") + raw.startswith(b">")
    assert np.array_equal(rs, run_start) and np.array_equal(rq, run_seq) and np.array_equal(rp, run_seqpos)
    assert all(raw[int(p)] == ord(">") for p in hp)
    low = bases | 0x20
    assert [int(x) for x in nucl] == [int(np.count_nonzero(low == ord(c))) for c in "acgt"]
    P, lens, thr = make_bank(60 + seed, 24, 5, 20, rel=0.8)
    scanner.set_mode("auto")
    scanner.set_motifs(P, lens, thr)
    whole = oracle.scan(bases, run_start, P, lens, thr)
    payload, overlap = 7_001, int(lens.max()) - 1
    parts = []
    for begin in range(0, nb, payload):
        size = min(payload + overlap, nb - begin)
        h = scanner.scan_stream(begin, size, _chunk_runs(run_start, begin, size))
        h = h[h["pos"] < payload]
        h["pos"] += begin
        parts.append(h)
    ok, msg = same_hits(np.concatenate(parts), whole)
    assert ok, msg
    assert len(whole) > 100


def test_resident_stream_rejects_positions_outside_it(scanner):
    from blamm_gb300 import BlammError
    from bankutil import make_bank
    scanner.stream_load_fasta(b">s\nACGTACGTAC\n")
    P, lens, thr = make_bank(5, 2, 3, 4)
    scanner.set_motifs(P, lens, thr)
    with pytest.raises(BlammError):
        scanner.scan_stream(4, 7, np.zeros(1, dtype=np.int64))
    assert len(scanner.scan_stream(4, 6, np.zeros(1, dtype=np.int64), hit_cap=1000)) >= 0
