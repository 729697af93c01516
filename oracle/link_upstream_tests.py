"""Compile the upstream NQS unit tests (tests/test_nqs*.c of the reference, read where they
lie) against this repository's include/ and link them against libnqs_gb300.so.

A test file that compiles and links unchanged shows that every upstream symbol and
signature it uses is provided by the drop-in; the binaries land in oracle/_ref/linkcheck/
(git-ignored, like the rest of oracle/_ref).  They need a GPU to run.  Prints one JSON
object {test name: "links" | "compile: <first error>" | "link: <missing symbols>"}.
Usage: python oracle/link_upstream_tests.py [reference root]
"""
import glob
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref", "linkcheck")
LIBDIR = os.path.join(ROOT, "spin_based_neural_network_gb300")


def default_reference():
    """Root of the upstream checkout: $NQS_REFERENCE_SRC, else the root that oracle/Makefile
    recorded when it built oracle/_ref (None when neither is set)."""
    env = os.environ.get("NQS_REFERENCE_SRC")
    if env:
        return env
    rec = os.path.join(HERE, "_ref", "source_root.txt")
    if os.path.exists(rec):
        with open(rec) as f:
            return f.read().strip() or None
    return None


def check(ref):
    os.makedirs(OUT, exist_ok=True)
    res = {}
    for src in sorted(glob.glob(os.path.join(ref, "tests", "test_nqs*.c"))):
        name = os.path.basename(src)[:-2]
        obj, exe = os.path.join(OUT, name + ".o"), os.path.join(OUT, name)
        c = subprocess.run(["gcc", "-std=c11", "-D_GNU_SOURCE", "-O0", "-I" + os.path.join(ROOT, "include"),
                            "-I" + os.path.join(ref, "tests"), "-c", src, "-o", obj], capture_output=True, text=True)
        if c.returncode:
            err = next((l for l in c.stderr.splitlines() if "error" in l), c.stderr.strip()[:160])
            res[name] = "compile: " + err.split("error:")[-1].strip()
            continue
        l = subprocess.run(["gcc", "-o", exe, obj, "-L" + LIBDIR, "-lnqs_gb300", "-lm",
                            "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
        if l.returncode:
            missing = sorted(set(re.findall(r"undefined reference to `([A-Za-z_0-9]+)'", l.stderr)))
            res[name] = "link: " + " ".join(missing)
        else:
            res[name] = "links"
    return res


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else default_reference()
    if not ref:
        raise SystemExit("usage: link_upstream_tests.py <root of the upstream checkout> "
                         "(or set NQS_REFERENCE_SRC, or build oracle/_ref with make -C oracle REF=...)")
    print(json.dumps(check(ref), indent=1))
