"""The allocation interposer (libgbxblas_preload.so) under LD_PRELOAD.

CPU tests run with GBX_TRACKER_FAKE_MANAGED=1 (host memory stands in for
managed memory, no CUDA call is made) and check the placement decisions, the
oracle-file workflow, realloc/calloc/free semantics, alignment and thread
safety.  The GPU test runs dgemm_ on operands the interposer placed in real
managed memory and checks they are used in place (placement hits, no copies).
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PRELOAD = os.path.join(ROOT, "libgpublas_gb300", "libgbxblas_preload.so")
PROG_SRC = os.path.join(ROOT, "tests", "tracker_prog.c")


@pytest.fixture(scope="module")
def prog(lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("tracker") / "tracker_prog")
    subprocess.check_call(["gcc", "-O1", "-o", exe, PROG_SRC, "-ldl", "-lpthread"])
    return exe


def run(prog, args, options="", fake=True, cwd=None):
    env = dict(os.environ)
    env["LD_PRELOAD"] = PRELOAD
    env["BLAS2CUDA_OPTIONS"] = options
    if fake:
        env["GBX_TRACKER_FAKE_MANAGED"] = "1"
    else:
        env.pop("GBX_TRACKER_FAKE_MANAGED", None)
    r = subprocess.run([prog] + args, capture_output=True, text=True, env=env, timeout=300, cwd=cwd)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    return r.stdout.splitlines()


def parse_seq(lines):
    objs = [tuple(int(v) for v in ln.split()) for ln in lines if ln[0].isdigit()]
    extra = {ln.split()[0]: [int(v) for v in ln.split()[1:]] for ln in lines if not ln[0].isdigit()}
    return objs, extra


def test_heuristic_false_keeps_everything_on_host(prog):
    objs, extra = parse_seq(run(prog, ["seq"], "heuristic=false"))
    assert len(objs) == 10
    assert all(m == 0 for _, m, _ in objs)
    # indices are consecutive: every malloc/calloc of the program is counted
    nths = [n for n, _, _ in objs]
    assert nths == list(range(nths[0], nths[0] + 10))


def test_heuristic_true_places_everything_managed_aligned(prog):
    objs, extra = parse_seq(run(prog, ["seq"], "heuristic=true"))
    assert all(m == 1 and al == 1 for _, m, al in objs)
    assert extra["objects_after_free"][0] == 0
    assert extra["memalign"][:2] == [1, 1]


def test_managed_min_threshold(prog):
    objs, _ = parse_seq(run(prog, ["seq"], "heuristic=true;managed_min=4096"))
    sizes = [16, 300, 4096, 100000, 3 << 20, 64, 1 << 20, 777, 5000, 65536]
    assert [m for _, m, _ in objs] == [int(s >= 4096) for s in sizes]


def test_oracle_file_selects_exact_objects(prog, tmp_path):
    base, _ = parse_seq(run(prog, ["seq"], "heuristic=false"))
    nths = [n for n, _, _ in base]
    chosen = {nths[1], nths[4], nths[8]}
    lines = []
    for i, n in enumerate(nths):
        tag = "D" if n in chosen else "H"
        lines.append(f"{tag} #{n} U{i} fun=[malloc] reqsize=[100] alive=(0, None)")
    lines.append("garbage line that does not parse")
    f = tmp_path / "trace.txt"
    f.write_text("\n".join(lines) + "\n")
    objs, _ = parse_seq(run(prog, ["seq"], f"heuristic=oracle:{f}"))
    assert [n for n, _, _ in objs] == nths
    assert {n for n, m, _ in objs if m} == chosen


def test_oracle_file_missing_aborts(prog, tmp_path):
    env = dict(os.environ, LD_PRELOAD=PRELOAD, GBX_TRACKER_FAKE_MANAGED="1",
               BLAS2CUDA_OPTIONS=f"heuristic=oracle:{tmp_path / 'nope.txt'}")
    r = subprocess.run([prog, "seq"], capture_output=True, text=True, env=env, timeout=60)
    assert r.returncode != 0 and "failed to load allocation oracle" in r.stderr


def test_random_heuristic_is_a_fair_coin(prog):
    # the reference's coin, random()/LONG_MAX > 0.5, never comes up on LP64
    # (obj_tracker.c:236); here about half of 2000 objects are managed
    managed, total = (int(v) for v in run(prog, ["many"], "heuristic=random")[-1].split()[1:3])
    assert total == 2000 and 800 <= managed <= 1200


def test_realloc_calloc_free_semantics(prog):
    lines = run(prog, ["realloc"], "heuristic=true")
    d = {ln.split()[0]: [int(v) for v in ln.split()[1:]] for ln in lines}
    assert d["realloc"] == [111, 11, 1]      # zeroed calloc, managed before/after, content kept
    assert d["reuse"] == [1, 1, 0]           # freed block is reused
    assert d["realloc_null"][0] == 1


@pytest.mark.parametrize("options", ["heuristic=true", "heuristic=random", "heuristic=false"])
def test_threads_stress(prog, options):
    lines = run(prog, ["threads"], options)
    bad, objs, nbytes = (int(v) for v in lines[-1].split()[1:])
    # at most the C library's per-thread records (one per thread) remain;
    # the workers' objects (up to 200 kB each) are all freed
    assert bad == 0 and objs <= 8 and nbytes <= 8 * 4096


def test_statistics_file(prog, tmp_path):
    f = tmp_path / "stats.csv"
    run(prog, ["seq"], f"heuristic=true;statistics={f}")
    head, vals = f.read_text().splitlines()
    row = dict(zip(head.split(","), (int(v) for v in vals.split(","))))
    assert row["managed_objects"] == 0 and row["counted_allocs"] >= 10


def test_trace_to_decision_file_workflow(prog, tmp_path):
    # producer: trace a run; analyze: objects named by BLAS calls become "D";
    # consumer: rerun with the decision file, exactly those are managed.
    import sys
    trace = tmp_path / "run.trace"
    dec = tmp_path / "decisions.txt"
    lines = run(prog, ["blas_note"], f"heuristic=false;errors=return;trace={trace}")
    assert [ln.split()[1] for ln in lines] == ["0"] * 6
    text = trace.read_text()
    assert text.count("fun=[dgemm_]") == 3 and text.count("\nU #") + text.startswith("U #") >= 6
    r = subprocess.run([sys.executable, "-m", "libgpublas_gb300.analyze_trace", str(trace), str(dec)],
                       capture_output=True, text=True, cwd=ROOT, timeout=60)
    assert r.returncode == 0, r.stderr
    d_lines = [ln for ln in dec.read_text().splitlines() if ln.startswith("D ")]
    assert len(d_lines) == 3
    lines = run(prog, ["blas_note"], f"heuristic=oracle:{dec};errors=return")
    assert [int(ln.split()[1]) for ln in lines] == [0, 1, 0, 1, 1, 0]


@pytest.mark.gpu
def test_managed_operands_are_used_in_place(prog):
    # real managed memory: dgemm_ on operands the interposer placed there is a
    # placement hit for every operand and moves no bytes through staging
    lines = run(prog, ["blas", "512"], "heuristic=true;managed_min=65536", fake=False)
    d = {" ".join(ln.split()[:2]): [int(v) for v in ln.split()[2:]] for ln in lines}
    assert d["blas managed"] == [1, 1, 1]
    hits, misses, moved = d["blas stats"]
    assert hits == 3 and misses == 0 and moved == 0
    lines = run(prog, ["blas", "512"], "heuristic=false", fake=False)
    d = {" ".join(ln.split()[:2]): [int(v) for v in ln.split()[2:]] for ln in lines}
    assert d["blas managed"] == [0, 0, 1]
    hits, misses, moved = d["blas stats"]
    assert hits == 0 and misses == 3 and moved > 0


# ---- OBJTRACKER_OPTIONS and the runnable library (lib/obj_tracker.c:246-321,
# entry.c:4-11); all on the CPU: forwarded calls never reach the GPU path
@pytest.fixture(scope="module")
def fake_blas(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("fakeblas") / "libfakecpublas.so")
    subprocess.check_call(["gcc", "-O1", "-shared", "-fPIC", "-o", so,
                           os.path.join(ROOT, "tests", "fake_cpublas.c"), "-lm"])
    return so


def run_env(prog, args, options="", objtracker=None):
    env = dict(os.environ, LD_PRELOAD=PRELOAD, BLAS2CUDA_OPTIONS=options, GBX_TRACKER_FAKE_MANAGED="1")
    if objtracker is not None:
        env["OBJTRACKER_OPTIONS"] = objtracker
    return subprocess.run([prog] + args, capture_output=True, text=True, env=env, timeout=300)


def test_blas_libs_forwards_calls_to_the_named_library(prog, fake_blas, tmp_path):
    trace = tmp_path / "fwd.trace"
    r = run_env(prog, ["fwd"], f"heuristic=false;errors=return;trace={trace}", f"blas_libs={fake_blas}")
    assert r.returncode == 0, r.stderr
    res = {ln.split()[0]: int(ln.split()[1]) for ln in r.stdout.splitlines()}
    assert res == {"dgemm": 1, "dsymm": 1, "ddot": 30, "idamax": 3}, r.stdout
    for name in ("dgemm_", "dsymm_", "ddot_", "idamax_"):
        assert f"fake {name}" in r.stderr
    assert "gbxblas:" not in r.stderr          # nothing ran (or failed) on the GPU path
    text = trace.read_text()
    # the traced program's objects and the calls naming them are all recorded
    assert text.count("\nC #") + text.startswith("C #") == 3 + 3 + 2 + 1
    assert "T #" in text


def test_only_print_calls_keeps_the_call_lines(prog, fake_blas, tmp_path):
    import sys
    trace = tmp_path / "calls.trace"
    r = run_env(prog, ["fwd"], f"heuristic=false;trace={trace}", f"only_print_calls;blas_libs={fake_blas}")
    assert r.returncode == 0, r.stderr
    lines = trace.read_text().splitlines()
    assert lines and all(ln.startswith("C #") for ln in lines)
    dec = tmp_path / "dec.txt"
    a = subprocess.run([sys.executable, "-m", "libgpublas_gb300.analyze_trace", str(trace), str(dec)],
                       capture_output=True, text=True, cwd=ROOT, timeout=60)
    assert a.returncode == 0, a.stderr
    d = [ln for ln in dec.read_text().splitlines() if ln.startswith("D #")]
    assert len(d) == 3                          # a, b, c: every object a call named


def test_objtracker_help_debug_uninit_and_unknown_option(prog):
    r = run_env(prog, ["seq"], "heuristic=false", "help;debug_uninit;no_such_option")
    assert r.returncode == 0, r.stderr
    assert "object tracker options" in r.stderr and "blas_libs" in r.stderr
    assert "before initialisation" in r.stderr
    assert "unknown option 'no_such_option'" in r.stderr


def test_missing_blas_library_aborts(prog, tmp_path):
    r = run_env(prog, ["seq"], "heuristic=false", f"blas_libs={tmp_path / 'nope.so'}")
    assert r.returncode != 0 and "dlopen" in r.stderr


def test_running_the_library_prints_its_options(lib):
    blas = os.path.join(ROOT, "libgpublas_gb300", "libgbxblas.so")
    r = subprocess.run([blas], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "BLAS2CUDA_OPTIONS" in r.stdout, (r.returncode, r.stdout, r.stderr)
    r = subprocess.run([PRELOAD], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "BLAS2CUDA_OPTIONS" in r.stdout and "OBJTRACKER_OPTIONS" in r.stderr


def test_side_table_under_churn(prog):
    # freed entries leave no tombstones: after 300k allocate/free pairs the
    # table holds exactly the live objects, probe runs stay short, and
    # interior pointers are never mistaken for objects
    lines = run(prog, ["churn"], "heuristic=true")
    d = {ln.split()[0]: [int(v) for v in ln.split()[1:]] for ln in lines}
    live, used, bad = d["live"]
    assert used == live and bad == 0
    assert d["after"][0] == 0 and d["after"][1] == 0


def test_posix_memalign_rejects_bad_alignment(prog):
    import errno
    for options in ("heuristic=true", "heuristic=false"):
        d = {ln.split()[0]: [int(v) for v in ln.split()[1:]] for ln in run(prog, ["align"], options)}
        assert d["posix_memalign"] == [errno.EINVAL, errno.EINVAL, 1]
        assert d["memalign"][:2] == [1, 1]
