"""Host side (C++ libblamm_host.so + the `blamm` CLI without a GPU) against the oracle
and the reference's golden files."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import golden_cases as gc
import oracle
from blamm_gb300 import workloads
from blamm_gb300._native import CLI_PATH, FastaReader, MotifBank

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the command line without a GPU: its host FASTA reader (the default reader parses on the GPU)
HOST_READER = {"BLAMM_FASTA_READER": "host"}
HOST_ENV = dict(os.environ, **HOST_READER)


@pytest.mark.parametrize("case", gc.CASES)
def test_cli_dict_and_hist_match_reference(tmp_path, case):
    spec = gc.load(case)
    d = gc.stage(case, str(tmp_path))
    gc.run(CLI_PATH, d, spec, skip=[lambda c: c[0] == "scan", lambda c: c[0] == "hist" and "-e" in c],
           env=HOST_READER)
    gc.compare(d, case, spec, what=("dict", "hist"))


def _pfms(seed, n, lmin, lmax):
    return [p for _, p in workloads.random_pfms(np.random.default_rng(seed), n, lmin, lmax)]


def test_bank_matrix_equals_oracle_pwms():
    pf = _pfms(31, 40, 4, 30)
    bank = MotifBank.from_pfms(pf, revcompl=True)
    bg = [12345, 6789, 7000, 13000]
    bank.generate(bg, 0.25)
    P, lens, rc = bank.matrix()
    order = sorted(range(len(pf)), key=lambda i: pf[i].shape[0])
    # the container is sorted by length (std::sort; equal lengths may permute), so match by content
    cols = []
    for i in order:
        cols.append((oracle.pfm2pwm(pf[i], bg, 0.25, False), 0))
        cols.append((oracle.pfm2pwm(oracle.revcompl_pfm(pf[i]), bg, 0.25, True), 1))
    got = {(P[c, :4 * lens[c]].tobytes(), int(rc[c])) for c in range(P.shape[0])}
    want = {(w.tobytes(), r) for w, r in cols}
    assert got == want
    assert np.all(np.diff(lens) >= 0)
    assert np.all(rc[1::2] == 1) and np.all(rc[0::2] == 0)
    mn, mx = bank.min_max()
    for c in range(P.shape[0]):
        omn, omx = oracle.min_max_score(P[c, :4 * lens[c]].reshape(-1, 4))
        assert (mn[c], mx[c]) == (np.float32(omn), np.float32(omx))


def test_bank_pvalue_thresholds_equal_oracle():
    pf = _pfms(32, 12, 5, 25)
    bank = MotifBank.from_pfms(pf, revcompl=True)
    counts = [2900, 2100, 2100, 2900]
    bank.generate(counts, 0.25)
    P, lens, rc = bank.matrix()
    bgp = oracle.nucl_prob(counts, 0.25)
    thr = bank.pvalue_thresholds(bgp, 1e-4, 250, 10_000_000)
    for c in range(0, P.shape[0], 2):  # forward columns; rc columns share the threshold
        pwm = P[c, :4 * lens[c]].reshape(-1, 4)
        mn, mx = oracle.min_max_score(pwm)
        width = np.float32(np.float32(mx) - np.float32(mn)) / np.float32(250)
        h = oracle.theoretical_hist(pwm, bgp, 250, 10_000_000)
        want = oracle.score_cutoff(h, mn, float(width), mx, 1e-4)
        assert np.float32(thr[c]) == np.float32(want) and thr[c + 1] == thr[c]


def _oracle_stream(files, max_filt=-1):
    """orc_stream_read through ctypes: (bases, run_start, run_seq, run_seqpos, names)."""
    L = oracle.lib()

    class S(C.Structure):
        _fields_ = [("bases", C.c_void_p), ("n", C.c_int64), ("run_start", C.c_void_p),
                    ("run_seq", C.c_void_p), ("run_seqpos", C.c_void_p), ("nruns", C.c_int64),
                    ("names", C.c_void_p), ("nseq", C.c_int64), ("tot_seq_len", C.c_int64)]
    L.orc_stream_read.argtypes = [C.POINTER(C.c_char_p), C.c_int, C.c_int64, C.POINTER(S), C.c_char_p, C.c_int]
    L.orc_stream_free.argtypes = [C.POINTER(S)]
    s = S()
    err = C.create_string_buffer(512)
    arr = (C.c_char_p * len(files))(*[f.encode() for f in files])
    assert L.orc_stream_read(arr, len(files), max_filt, C.byref(s), err, 512) == 0, err.value
    def a64(p, k):
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int64)), (k,)).copy() if k else np.zeros(0, np.int64)
    bases = np.ctypeslib.as_array(C.cast(s.bases, C.POINTER(C.c_uint8)), (s.n,)).copy() if s.n else np.zeros(0, np.uint8)
    out = (bases, a64(s.run_start, s.nruns), a64(s.run_seq, s.nruns), a64(s.run_seqpos, s.nruns))
    L.orc_stream_free(C.byref(s))
    return out


@pytest.mark.parametrize("payload,overlap", [(10_000_000, 29), (997, 29), (4096, 0), (50, 23)])
@pytest.mark.parametrize("max_filt", [-1, 30_001])
def test_fasta_chunks_equal_oracle_stream(payload, overlap, max_filt):
    files = [os.path.join(gc.GOLDEN, "mixed", "seqs", f) for f in ("a_file.fa", "b_file.fa")]
    _check_chunks(files, payload, overlap, max_filt)


@pytest.mark.parametrize("crlf", [False, True])
def test_fasta_edge_cases_stream_like_the_oracle(tmp_path, crlf):
    """A header without bases, a 3-base sequence, IUPAC codes, no final newline, CRLF."""
    from fresh_cases import edge_case
    edge_case(tmp_path, crlf)
    files = [str(tmp_path / "a.fa")]
    for payload, overlap in ((10_000_000, 15), (997, 15), (64, 0)):
        _check_chunks(files, payload, overlap, -1)
    rd = FastaReader(files, -1)
    while rd.next_chunk(1 << 20, 15) is not None:
        pass
    assert rd.sequence_names() == ["empty", "short", "iupac", "last"]


@pytest.mark.skipif(not os.path.exists(oracle.REF_CLI_PATH), reason="reference binary only in the development container")
@pytest.mark.parametrize("kind,arg", [("edge", False), ("edge", True), ("random", 0), ("random", 1)])
def test_cli_dict_and_hist_match_reference_on_fresh_cases(tmp_path, kind, arg):
    """FASTA edge cases (LF, CRLF) and seeded random cases (two species groups, N runs,
    soft-masked stretches, JASPAR and Cluster-Buster motifs)."""
    import subprocess
    from fresh_cases import edge_case, random_case
    make = edge_case if kind == "edge" else random_case
    outs = {}
    for name, binary in (("ref", oracle.REF_CLI_PATH), ("ours", CLI_PATH)):
        d = tmp_path / name
        d.mkdir()
        cmds = [c for c in make(d, arg) if c[0] != "scan"]
        for cmd in cmds:
            subprocess.run([binary] + cmd, cwd=d, check=True, stdout=subprocess.DEVNULL,
                           env=dict(HOST_ENV, OPENBLAS_NUM_THREADS="1"))
        outs[name] = d
    files = ["sequences.mf.dict"] + sorted(p.name for p in outs["ref"].glob("hist_*"))
    assert len(files) > 1
    for f in files:
        assert (outs["ref"] / f).read_bytes() == (outs["ours"] / f).read_bytes(), f


def _check_chunks(files, payload, overlap, max_filt):
    """The C++ reader's chunks against the oracle's stream of the same files."""
    bases, rs, rq, rp = _oracle_stream(files, max_filt)
    rd = FastaReader(files, max_filt)
    pos = 0
    while True:
        ch = rd.next_chunk(payload, overlap)
        if ch is None:
            break
        off, pay, b, mk = ch
        assert off == pos
        assert np.array_equal(b, bases[off:off + len(b)])
        assert len(b) == min(payload + overlap, len(bases) - off) and pay == min(payload, len(b))
        # every chunk position maps to the same (sequence, position) as in the oracle's stream
        r = np.searchsorted(rs, off + mk[:, 0], side="right") - 1
        assert np.array_equal(rq[r], mk[:, 1])
        assert np.array_equal(rp[r] + (off + mk[:, 0] - rs[r]), mk[:, 2])
        # markers inside the chunk are exactly the oracle's run starts there
        inside = rs[(rs > off) & (rs < off + len(b))] - off
        assert np.array_equal(mk[1:, 0], inside) and mk[0, 0] == 0
        pos += pay
    assert pos == len(bases)


def test_every_declared_symbol_is_exported():
    from blamm_gb300._native import gpu_lib, host_lib
    for header, lib in (("blamm_gpu.h", gpu_lib()), ("blamm_host.h", host_lib()), ("blamm_serve.h", host_lib())):
        text = open(os.path.join(ROOT, "include", header)).read()
        names = set(re.findall(r"^[A-Za-z_][\w \*]*?\b(blamm_\w+)\s*\(", text, flags=re.M))
        assert len(names) > 5
        for name in sorted(names):
            assert hasattr(lib, name), f"{header}: {name} is not exported"


def test_genome_parts_share_the_bank_and_not_the_bases():
    """The parts the benchmark's ranks scan at N > 1: one motif bank, distinct sequences;
    part 0 is the single-GPU workload itself."""
    a = workloads.genome_100mbp(0, total=300_000, nseq=4)
    a0 = workloads.genome_100mbp(0, total=300_000, nseq=4, part=0)
    b = workloads.genome_100mbp(0, total=300_000, nseq=4, part=1)
    assert all(np.array_equal(x[1], y[1]) for x, y in zip(a.motifs, b.motifs))
    assert all(np.array_equal(x[1], y[1]) for x, y in zip(a.sequences, a0.sequences))
    assert [s for s, _ in a.sequences] == ["chr1", "chr2", "chr3", "chr4"]
    assert [s for s, _ in b.sequences] == ["chr5", "chr6", "chr7", "chr8"]
    assert abs(b.total_bases - 300_000) <= 4
    assert not np.array_equal(a.sequences[0][1][:1000], b.sequences[0][1][:1000])


CUDA_INCLUDE = "/usr/local/cuda/include"


def test_integration_stub_compiles_against_the_reference(tmp_path):
    """The replacement body of PWMScan::scanThreadCUBLAS (tests/integration_stub.cpp) compiles
    (syntax and types) against the reference's unmodified headers and include/blamm_gpu.h."""
    import shutil
    import subprocess
    import oracle_build
    ref_src = os.path.join(oracle_build.reference_dir(), "src")
    if not os.path.isdir(ref_src) or not os.path.isdir(CUDA_INCLUDE) or not shutil.which("g++"):
        pytest.skip("needs the reference's sources, the CUDA headers and g++")
    src = os.path.join(ROOT, "tests", "integration_stub.cpp")
    body = open(src).read()
    assert "blamm_scan(" in body and "getNextOverlappingBlock" in body
    # the reference's build generates config.h (F77 name mangling); any definition will do here
    (tmp_path / "config.h").write_text("#define F77_FUNC(name,NAME) name ## _\n")
    cmd = ["g++", "-std=c++11", "-fsyntax-only", "-Wall", "-DHAVE_CONFIG_H", "-DHAVE_CUDA",
           f"-I{tmp_path}", f"-I{ref_src}", f"-I{os.path.join(ROOT, 'include')}", f"-I{CUDA_INCLUDE}"]
    # the reference's headers use these without including them under gcc 13
    for h in ("array", "mutex", "cassert", "limits", "stdexcept", "map", "future"):
        cmd += ["-include", h]
    r = subprocess.run(cmd + [src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_cli_errors_match_reference_behaviour(tmp_path):
    """Host-side failures: missing files give a message and EXIT_FAILURE like the reference."""
    import subprocess
    d = gc.stage("cb", str(tmp_path))
    r = subprocess.run([CLI_PATH, "dict", "missing.mf"], cwd=d, capture_output=True, env=HOST_ENV)
    assert r.returncode == 1 and b"Could not open file: missing.mf" in r.stderr
    r = subprocess.run([CLI_PATH, "hist", "motifs.cb", "sequences.mf"], cwd=d, capture_output=True)
    assert r.returncode == 1 and b"Cannot open file: sequences.mf.dict" in r.stderr
    r = subprocess.run([CLI_PATH, "scan", "-rt", "0.9", "-at", "3", "motifs.cb", "sequences.mf"], cwd=d,
                       capture_output=True)
    assert r.returncode == 1 and b"not both" in r.stderr
    r = subprocess.run([CLI_PATH, "scan", "-pt", "2", "motifs.cb", "sequences.mf"], cwd=d, capture_output=True)
    assert r.returncode == 1 and b"p-value should be in range" in r.stderr
    with open(os.path.join(d, "bad.fa"), "w") as f:
        f.write("ACGT\n>x\nACGT\n")
    with open(os.path.join(d, "bad.mf"), "w") as f:
        f.write("sp\tbad.fa\n")
    r = subprocess.run([CLI_PATH, "dict", "bad.mf"], cwd=d, capture_output=True, env=HOST_ENV)
    assert r.returncode == 1 and b"does not appear to be in fasta format" in r.stderr


def test_bank_hist_columns_map_rc_columns_to_their_forward_motif():
    """blamm_bank_hist_columns: each column's histogram comes from its forward motif
    (the same base name), as the reference's hist files are named (src/motif.h:256-267)."""
    rng = np.random.default_rng(12)
    pf = [p for _, p in workloads.random_pfms(rng, 20, 5, 15)]
    bank = MotifBank.from_pfms(pf, revcompl=True)
    bank.generate(np.array([30, 20, 20, 30], dtype=np.uint64), 0.25)
    _, _, rc = bank.matrix()
    hof = bank.hist_columns()
    for c in range(bank.columns):
        h = int(hof[c])
        assert rc[h] == 0 and bank.name(h) == bank.name(c).replace("_rc", "")[: len(bank.name(h))]
        if rc[c] == 0:
            assert h == c


def test_cli_rejects_sequence_data_before_a_header(tmp_path):
    """A FASTA file whose first line is sequence data: the same message and exit code as the
    reference's dict module (FastaBatch::getNextLine throws, blstools.cpp:93-101 exits 1)."""
    import subprocess
    (tmp_path / "bad.fa").write_text("ACGT\n>s1\nACGTACGT\n")
    (tmp_path / "bad.mf").write_text("sp\tbad.fa\n")
    r = subprocess.run([CLI_PATH, "dict", "bad.mf"], cwd=tmp_path, capture_output=True, env=HOST_ENV)
    assert r.returncode == 1
    assert b"Input file does not appear to be in fasta format" in r.stderr + r.stdout


def test_score_text_equals_printf_g():
    """The occurrence-file score formatter against printf("%g") (the reference's default
    ostream output): a whole binade exhaustively, random magnitudes and signs, decimal
    ties, carries to the next power of ten, and the values outside the fast path."""
    from blamm_gb300._native import format_scores
    rng = np.random.default_rng(7)
    binade = (np.arange(1 << 23, dtype=np.uint32) | np.uint32(0x3F800000)).view(np.float32)  # [1, 2)
    rand_mag = (np.exp(rng.uniform(np.log(1e-7), np.log(1e9), 2_000_000)) *
                rng.choice([-1.0, 1.0], 2_000_000)).astype(np.float32)
    scores = rng.uniform(-60, 40, 1_000_000).astype(np.float32)
    ties = np.array([float(f"{d}.{x:05d}5") for d in range(1, 10) for x in range(0, 100000, 997)],
                    dtype=np.float32)
    edges = np.array([9.999995, 99999.95, 999999.5, 1e-4, 9.99999e-5, 1e6, 0.0, -0.0, 123456.5, 0.5,
                      np.inf, -np.inf, np.nan, 1e-40, 3.4e38], dtype=np.float32)
    for v in (binade, rand_mag, scores, ties, edges):
        got = format_scores(v)
        want = oracle.format_scores(v)
        bad = [i for i, (g, w) in enumerate(zip(got, want)) if g != w]
        assert not bad, [(float(v[i]), got[i], want[i]) for i in bad[:5]]


def test_bench_reference_arm_prints_the_contract_line():
    """bench.py --impl reference (the reference's CPU algorithm, oracle port) prints one JSON
    line with the keys the benchmark contract names, on a small workload."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--bases",
                          "2000000", "--cpu-sample", "50000", "--steps", "1", "--warmup", "3"],
                         cwd=root, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    # the arm runs the oracle only: no product library in the process
    assert line["product_libraries_loaded"] == []
    assert line["sample_hits"]["hits"] > 0
    assert line["cli_e2e"]["value"] > 0 and line["cli_e2e"]["occurrence_lines"] > 0


def test_oracle_bank_equals_product_bank():
    """The oracle's restatement of the reference's scan set-up (used by the benchmark's
    reference arm) gives the product's motif bank: per (PFM, strand) the same PWM bits, length
    and p-value thresholds."""
    from blamm_gb300 import workloads
    rng = np.random.default_rng(5)
    pfms = [p for _, p in workloads.random_pfms(rng, 40, 5, 30)]
    counts = np.array([2900, 2100, 2100, 2900], dtype=np.uint64)
    P, lens, thr, cmot, cstr = oracle.motif_bank(pfms, counts, 0.25, (1e-4, 1e-5))
    bank = MotifBank.from_pfms(pfms, revcompl=True)
    bank.generate(counts, 0.25)
    Pb, lb, rcb = bank.matrix()
    bgp = oracle.nucl_prob(counts, 0.25)
    tb = [bank.pvalue_thresholds(bgp, pv, 250, 10_000_000) for pv in (1e-4, 1e-5)]
    assert np.all(np.diff(lens) >= 0)
    got = {(int(cmot[c]), int(cstr[c])): (P[c, :4 * lens[c]].tobytes(), thr[0][c], thr[1][c])
           for c in range(len(lens))}
    want = {(int(bank.name(c)[1:]), int(rcb[c])): (Pb[c, :4 * lb[c]].tobytes(), tb[0][c], tb[1][c])
            for c in range(len(lb))}
    assert got == want


def _pieces(files, piece_bytes):
    L = C.CDLL(os.path.join(ROOT, "blamm_gb300", "_build", "libblamm_host.so"))
    L.blamm_fasta_pieces_open.argtypes = [C.POINTER(C.c_char_p), C.c_int, C.c_int64, C.POINTER(C.c_void_p)]
    L.blamm_fasta_pieces_next.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]
    L.blamm_fasta_pieces_close.argtypes = [C.c_void_p]
    h = C.c_void_p()
    arr = (C.c_char_p * len(files))(*[f.encode() for f in files])
    assert L.blamm_fasta_pieces_open(arr, len(files), piece_bytes, C.byref(h)) == 0
    out = []
    while True:
        t, n = C.c_void_p(), C.c_int64()
        rc = L.blamm_fasta_pieces_next(h, C.byref(t), C.byref(n))
        assert rc >= 0
        if rc == 0:
            break
        out.append(C.string_at(t, n.value))
    L.blamm_fasta_pieces_close(h)
    return out


@pytest.mark.parametrize("piece_bytes", [1, 7, 100, 5000, 1 << 26])
def test_fasta_pieces_cut_only_at_header_lines(tmp_path, piece_bytes):
    """The GPU reader's pieces: the files' text in order (a final newline added where a file
    lacks one), each piece but the last at least piece_bytes long and ending right before a
    header line, with no header line starting past piece_bytes inside it."""
    rng = np.random.default_rng(piece_bytes)
    files, want = [], b""
    for fi in range(5):
        parts = []
        if fi == 3:  # a file that continues the previous file's last sequence
            parts.append(b"ACGTNNacgt\n")
        for si in range(int(rng.integers(0, 4))):
            parts.append(f">f{fi}s{si} descr\n".encode())
            for _ in range(int(rng.integers(0, 5))):
                parts.append(rng.choice(np.frombuffer(b"ACGTacgtN", np.uint8), int(rng.integers(0, 90))).tobytes() + b"\n")
        text = b"".join(parts)
        if text and rng.random() < 0.5:
            text = text[:-1]  # no final newline
        p = tmp_path / f"f{fi}.fa"
        p.write_bytes(text)
        files.append(str(p))
        want += text + (b"\n" if text and not text.endswith(b"\n") else b"")
    got = _pieces(files, piece_bytes)
    assert b"".join(got) == want
    for i, piece in enumerate(got):
        if i > 0:
            assert piece.startswith(b">")
        if i < len(got) - 1:
            assert len(piece) >= piece_bytes and piece.endswith(b"\n")
            assert piece.find(b"\n>", max(0, piece_bytes - 1)) in (-1, len(piece) - 1)


def test_fasta_header_names_like_the_reference():
    """`iss >> name` on the header line after '>': leading blanks skipped, the name ends at
    the first blank (space, tab, CR); an empty header gives an empty name."""
    L = C.CDLL(os.path.join(ROOT, "blamm_gb300", "_build", "libblamm_host.so"))
    L.blamm_fasta_header_name.argtypes = [C.c_char_p, C.c_int64, C.c_int64, C.c_char_p, C.c_int]
    text = b">chr1 desc\nACGT\n>  \tchr2\tx\r\n>\n>chr3\r\nAC\n>last"
    pos = [i for i in range(len(text)) if text[i:i + 1] == b">" and (i == 0 or text[i - 1:i] == b"\n")]
    out = C.create_string_buffer(64)
    names = []
    for p in pos:
        n = L.blamm_fasta_header_name(text, len(text), p, out, 64)
        assert n >= 0
        names.append(out.value.decode())
    assert names == ["chr1", "chr2", "", "chr3", "last"]
