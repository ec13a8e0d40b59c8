"""The reference's own command-line programs (src/Exec-*.c) compile against
this repository's headers and link against libirwls_gb300.so unchanged; run
without arguments they print their usage and exit with status 4, as the
reference's do. Needs the reference sources, so it is skipped where they are
absent."""
import os
import subprocess
import tempfile

import pytest

import harness as H

REF = "/root/reference/src"
PROGRAMS = ["Exec-full-train", "Exec-budgeted-train", "Exec-LIBIRWLS-predict"]


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
@pytest.mark.parametrize("prog", PROGRAMS)
def test_reference_cli_relinks_unchanged(prog):
    libdir = os.path.join(H.ROOT, "libirwls_gb300")
    out = os.path.join(tempfile.mkdtemp(), prog)
    r = subprocess.run(["gcc", "-w", "-fopenmp", "-I" + os.path.join(H.ROOT, "include"),
                        os.path.join(REF, prog + ".c"), "-o", out, "-L" + libdir, "-l:libirwls_gb300.so",
                        "-Wl,-rpath," + libdir, "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([out], capture_output=True, text=True)
    assert run.returncode == 4
    assert "Usage" in run.stderr
