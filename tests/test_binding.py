"""The reference-side binding of INTEGRATION.md, compiled: the
``iterators_gb300.cpp`` listed there is built together with the reference's
own main.cpp, aux.cpp, grid.cpp, gilbert2d.cpp and iterators.cpp (read in
place, never copied), with ITERATE bound to ``iterate_gb300`` and linked
against libst3d.so.  Without a GB300 the resulting hstencil3d must stop at
its first ITERATE with the library's no-device error (exit status 3), never
computing on the CPU; on a machine with a GB300 it must pass the reference's
own known-answer check.  Needs the reference's sources (ST3D_REFERENCE_DIR)."""
import os
import re
import subprocess

import pytest

from oracle import build as obuild
from stencil3d_gb300 import build as pbuild

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def binding_source():
    """The C++ listing that follows the iterators_gb300.cpp heading line."""
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    m = re.search(r"`iterators_gb300\.cpp`.*?```cpp\n(.*?)```", text, flags=re.S)
    assert m, "INTEGRATION.md lists no iterators_gb300.cpp"
    return m.group(1)


@pytest.fixture(scope="module")
def hstencil3d_gb300(tmp_path_factory):
    ref = obuild.ref_source_dir()
    if ref is None:
        pytest.skip("the reference's sources are not given (ST3D_REFERENCE_DIR)")
    out = tmp_path_factory.mktemp("binding")
    src = out / "iterators_gb300.cpp"
    src.write_text(binding_source())
    lib_dir = os.path.dirname(pbuild.LIB)
    common = ["g++", "-O2", "-std=c++17", "-fopenmp", "-w", "-D__builtin_assume(x)=((void)0)",
              "-I", ref, "-I", os.path.join(REPO, "include")]
    # ITERATE defaults to iterate_3d (config.h:55-65); binding it without an
    # edit of config.h renames that symbol in the TUs that call or define
    # the GPU replacement.  iterators.cpp stays as it is: it still supplies
    # init_arrays and check (iterators.cpp:292-325).
    bind = ["-Diterate_3d=iterate_gb300"]
    objs = []
    for f, extra in [(os.path.join(ref, "main.cpp"), bind), (os.path.join(ref, "aux.cpp"), []),
                     (os.path.join(ref, "grid.cpp"), []), (os.path.join(ref, "gilbert2d.cpp"), []),
                     (os.path.join(ref, "iterators.cpp"), []), (str(src), bind)]:
        o = out / (os.path.basename(f) + ".o")
        subprocess.run(common + extra + ["-c", f, "-o", str(o)], check=True)
        objs.append(str(o))
    exe = out / "hstencil3d_gb300"
    subprocess.run(["g++", "-fopenmp", "-o", str(exe)] + objs +
                   ["-L", lib_dir, "-lst3d", "-Wl,-rpath," + lib_dir], check=True)
    return str(exe)


def _gpu_visible():
    import stencil3d_gb300 as S
    try:
        S.device_info()
        return True
    except S.St3dError:
        return False


def test_binding_links_the_library(hstencil3d_gb300):
    out = subprocess.run(["nm", "-u", hstencil3d_gb300], capture_output=True, text=True,
                         check=True).stdout
    for sym in ("st3d_create", "st3d_iterate_host", "st3d_default_opts"):
        assert sym in out


def test_binding_runs_the_reference_driver(hstencil3d_gb300):
    r = subprocess.run([hstencil3d_gb300, "--xs", "32", "--ys", "32", "--zs", "32", "--iter", "2"],
                       capture_output=True, text=True, timeout=120,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    if _gpu_visible():
        assert r.returncode == 0, r.stderr
        assert "check: 0 errors found" in r.stdout
    else:
        # the reference driver's own output up to its first ITERATE, then the
        # library's refusal: no CPU computation stands in for the GPU
        assert "array initialization" in r.stdout
        assert r.returncode == 3, (r.returncode, r.stdout[-500:], r.stderr[-500:])
        assert "st3d_create" in r.stderr
