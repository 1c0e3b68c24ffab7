"""The ctypes mirrors of the C-ABI structs (nmag._lib) and of the oracle's
structs (oracle/oracle.py) have the C layout of their headers: size and
every field offset, from a small C program compiled with gcc against the
header.  CPU only."""
import ctypes
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def _structs():
    from nmag import _lib
    return [("nmg_material", _lib.Material), ("nmg_options", _lib.Options), ("nmg_ts_stats", _lib.TsStats),
            ("nmg_particle", _lib.Particle), ("nmg_batch_options", _lib.BatchOptions)]


def _oracle_structs():
    import oracle
    return [("om_mesh", oracle.OmMesh), ("om_material", oracle.OmMaterial), ("om_solver", oracle.OmSolver),
            ("om_state", oracle.OmState), ("om_ts_stats", oracle.OmStats)]


@pytest.mark.parametrize("which", ["library", "oracle"])
def test_ctypes_structs_match_the_header(tmp_path, which):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    header, incdir, structs = (("nmag_gpu.h", os.path.join(ROOT, "include"), _structs()) if which == "library"
                               else ("nmag_oracle.h", os.path.join(ROOT, "oracle"), _oracle_structs()))
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "%s"' % header, "int main(void) {"]
    for cname, cls in structs:
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in cls._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-I", incdir, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    c = {}
    for line in out:
        if line:
            a, b, v = line.split()
            c[(a, b)] = int(v)
    for cname, cls in structs:
        assert c[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert c[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
