"""The reference's own command-line programs (src/Exec-*.c) link against
libirwls_gb300.so unchanged; run without arguments they print their usage and
exit with status 4, as the reference's do.

Two forms, each skipped where its input is absent:
- from source: src/Exec-*.c of the reference checkout that the environment
  variable IRWLS_REFERENCE names, compiled against this repository's headers
  (the headers are a drop-in);
- from objects: oracle/_ref/Exec-*.o, which ``make -C oracle ref`` compiled
  from the same sources against the reference's own headers, linked against
  this library (the binary interface is a drop-in).
"""
import os
import subprocess
import tempfile

import pytest

import harness as H

REF = os.path.join(os.environ.get("IRWLS_REFERENCE", ""), "src") if os.environ.get("IRWLS_REFERENCE") else ""
OBJ = os.path.join(H.ROOT, "oracle", "_ref")
PROGRAMS = ["Exec-full-train", "Exec-budgeted-train", "Exec-LIBIRWLS-predict"]
LIBDIR = os.path.join(H.ROOT, "libirwls_gb300")
LINK = ["-L" + LIBDIR, "-l:libirwls_gb300.so", "-Wl,-rpath," + LIBDIR, "-lm"]


def _run_usage(exe):
    run = subprocess.run([exe], capture_output=True, text=True)
    assert run.returncode == 4
    assert "Usage" in run.stderr


@pytest.mark.skipif(not (REF and os.path.isdir(REF)), reason="IRWLS_REFERENCE does not name the reference sources")
@pytest.mark.parametrize("prog", PROGRAMS)
def test_reference_cli_source_relinks_unchanged(prog):
    out = os.path.join(tempfile.mkdtemp(), prog)
    r = subprocess.run(["gcc", "-w", "-fopenmp", "-I" + os.path.join(H.ROOT, "include"),
                        os.path.join(REF, prog + ".c"), "-o", out] + LINK, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _run_usage(out)


@pytest.mark.skipif(not all(os.path.exists(os.path.join(OBJ, p + ".o")) for p in PROGRAMS),
                    reason="the reference's objects are not built (make -C oracle ref)")
@pytest.mark.parametrize("prog", PROGRAMS)
def test_reference_cli_objects_link_unchanged(prog):
    out = os.path.join(tempfile.mkdtemp(), prog)
    r = subprocess.run(["gcc", "-fopenmp", os.path.join(OBJ, prog + ".o"), "-o", out] + LINK,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _run_usage(out)
