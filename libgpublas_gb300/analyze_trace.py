"""Turn an allocation/call trace into an allocation decision file.

The producer half of the allocation-file workflow (the reference's
scripts/objtrace.sh + scripts/analyze_trace.py): run the application once
with

    LD_PRELOAD=libgbxblas_preload.so BLAS2CUDA_OPTIONS="trace=run.trace" ./app

then

    python -m libgpublas_gb300.analyze_trace run.trace decisions.txt

and rerun with BLAS2CUDA_OPTIONS="heuristic=oracle:decisions.txt": every
object that a BLAS call named ("C" line) is placed in managed memory ("D"),
every other traced object stays on the host ("H").

Trace lines (written by the interposer):
  T #<nth> [<ptr>] fun=[malloc|calloc|realloc] reqsize=[<n>] tid=[..] time=[<s>s+<ns>ns] uid=[<uid>]
  U #<nth> ... fun=[free] ...
  C #<nth> ... fun=[<blas routine>] ...
(with OBJTRACKER_OPTIONS=only_print_calls only the C lines are written; the
decision file then lists the called objects alone, and the rest stay on the
host by default).
Decision lines:
  D #<nth> U<uid> fun=[malloc] reqsize=[<n>] calls=[<k>]
"""
import re
import sys

LINE = re.compile(r"^([TUC]) #(\d+) \[[^\]]*\] fun=\[(\w+)\] reqsize=\[(\d+)\].*uid=\[(\d+)\]")


def analyze(lines):
    """Returns {uid: dict(nth, fun, reqsize, calls)} from trace lines."""
    objs = {}
    for line in lines:
        m = LINE.match(line)
        if not m:
            continue
        kind, nth, fun, reqsize, uid = m.group(1), int(m.group(2)), m.group(3), int(m.group(4)), int(m.group(5))
        if kind == "T":
            objs[uid] = {"nth": nth, "fun": fun, "reqsize": reqsize, "calls": 0}
        elif kind == "C":
            # a trace written with OBJTRACKER_OPTIONS=only_print_calls has no
            # T lines: the call line carries the object's index and size
            o = objs.setdefault(uid, {"nth": nth, "fun": "alloc", "reqsize": reqsize, "calls": 0})
            o["calls"] += 1
    return objs


def decisions(objs):
    out = []
    for uid, o in sorted(objs.items(), key=lambda kv: kv[1]["nth"]):
        tag = "D" if o["calls"] else "H"
        out.append(f"{tag} #{o['nth']} U{uid} fun=[{o['fun']}] reqsize=[{o['reqsize']}] calls=[{o['calls']}]")
    return out


def main(argv):
    if len(argv) != 3:
        print(__doc__)
        return 2
    with open(argv[1]) as fh:
        objs = analyze(fh)
    lines = decisions(objs)
    with open(argv[2], "w") as fh:
        fh.write("\n".join(lines) + ("\n" if lines else ""))
    d = sum(1 for ln in lines if ln[0] == "D")
    print(f"{len(lines)} objects, {d} used by BLAS calls -> managed", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
