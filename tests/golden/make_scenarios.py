"""Golden output files of the scenario files in tests/golden/scenarios/,
written by the reference's own Solaris program (oracle/_ref/solaris, built
from the reference sources by oracle/Makefile).

For every <name>.xml the program runs in a scratch directory (it writes its
outputs next to the input file) and every output file but the time-stamped
log is copied to tests/golden/scenarios/<name>/.

    python tests/golden/make_scenarios.py [reference source root; default $SOLARIS_REFERENCE_SRC]
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SCENARIOS = os.path.join(HERE, "scenarios")


def main(ref_root=None):
    sys.path.insert(0, ROOT)
    import oracle
    ref_root = ref_root or oracle.REFERENCE_SRC
    if not oracle.build_reference(ref_root):
        raise SystemExit("the reference sources are not available")
    prog = os.path.join(oracle.REF_DIR, "solaris")
    for fn in sorted(os.listdir(SCENARIOS)):
        if not fn.endswith(".xml"):
            continue
        name = fn[:-4]
        with tempfile.TemporaryDirectory() as tmp:
            shutil.copy(os.path.join(SCENARIOS, fn), tmp)
            r = subprocess.run([prog, "-i", os.path.join(tmp, fn)], cwd=tmp, capture_output=True, text=True,
                               env=dict(os.environ, OSTYPE="linux"), timeout=600)
            if r.returncode != 0:
                raise SystemExit(f"{fn}: the reference program failed\n{r.stdout}\n{r.stderr}")
            out = os.path.join(SCENARIOS, name)
            shutil.rmtree(out, ignore_errors=True)
            os.makedirs(out)
            log = "Log.txt"
            for f in sorted(os.listdir(tmp)):
                if f == fn or f == log:
                    continue
                shutil.copy(os.path.join(tmp, f), out)
            print(name, sorted(os.listdir(out)))


if __name__ == "__main__":
    main(*sys.argv[1:])
