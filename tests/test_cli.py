"""gstencil3d, the hstencil3d-compatible driver: the argument handling of
main.cpp:123-174 and aux.cpp:16-81 (messages and exit codes), checked
against the reference binary where it was built on this machine.  No GPU:
a valid command line ends with exit status 3 (the library's no-device
error), never with a CPU computation."""
import os
import subprocess

import pytest

from oracle import build as obuild
from stencil3d_gb300 import build as pbuild

CLI = pbuild.CLI
REF = os.path.join(obuild.REF_DIR, "hstencil3d_7")


def run(exe, *args):
    r = subprocess.run([exe] + list(args), capture_output=True, text=True, timeout=60,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    return r.returncode, r.stdout, r.stderr


CASES = [
    (["--bogus"], 2, "unsupported argument --bogus"),
    (["--xh", "3"], 2, "--xh must be larger or equal to 4"),
    (["--xs", "2000"], 2, "--xs must be smaller or equal to 1264"),
    (["--iter"], 2, "--iter requires a numeric argument"),
    (["--ys", "10", "--yb", "3"], 2, "ERROR: --ys must by an exact multiple of --yb"),
    (["--sbm", "20"], 2, "--sbm must be smaller or equal to"),
]


@pytest.mark.parametrize("args,code,msg", CASES, ids=[" ".join(c[0]) for c in CASES])
def test_argument_errors_match_reference(args, code, msg):
    rc, out, err = run(CLI, *args)
    assert rc == code and msg in err
    if os.path.exists(REF):
        rrc, rout, rerr = run(REF, *args)
        assert rrc == code and msg in rerr


def test_flags_are_echoed_like_reference():
    rc, out, err = run(CLI, "--xs", "16", "--ys", "16", "--zs", "16", "--iter", "2", "--train")
    assert "--xs set to 16" in out and "--train set to ENABLED" in out
    assert "running STENCIL(7) benchmark" in out


def _gpu_visible():
    try:
        import stencil3d_gb300 as S
        S.device_info()
        return True
    except Exception:
        return False


@pytest.mark.skipif(_gpu_visible(), reason="a GPU is visible")
def test_no_device_is_an_error_not_a_fallback():
    rc, out, err = run(CLI, "--xs", "16", "--ys", "16", "--zs", "16", "--iter", "2")
    assert rc == 3
    assert "check:" not in out


@pytest.mark.gpu
@pytest.mark.parametrize("points", ["7", "13", "25"])
def test_known_answer_through_the_driver(points):
    """The reference's own known-answer run (main.cpp:289-312) on the GPU."""
    rc, out, err = run(CLI, "--xs", "48", "--ys", "40", "--zs", "160", "--iter", "5",
                       "--stencil", points)
    assert rc == 0, err
    assert out.count("check: 0 errors found") == 2
    assert "finish compute in" in out and "GFlop/s" in out and "Gpts/s" in out


@pytest.mark.gpu
def test_wave_form_through_the_driver():
    rc, out, err = run(CLI, "--xs", "40", "--ys", "40", "--zs", "128", "--iter", "10",
                       "--stencil", "25", "--wave", "--dt", "0.0005")
    assert rc == 0, err
    assert "leapfrog wave" in out and "finish compute in" in out


@pytest.mark.gpu
def test_vec16_variant_reproduces_the_reference_check():
    """--variant vec16 gives the 13-point kernel the reference's vec_16 K =
    6.25, whose known-answer check fails on every point (a step of -1.75
    instead of +1), as the reference's vec_16 build reports."""
    rc, out, err = run(CLI, "--xs", "16", "--ys", "16", "--zs", "32", "--iter", "2",
                       "--stencil", "13", "--variant", "vec16")
    assert rc == 0, err
    assert out.count("check: 8192 errors found") == 2
    rc, out, err = run(CLI, "--xs", "16", "--ys", "16", "--zs", "32", "--iter", "2",
                       "--stencil", "13", "--variant", "ref")
    assert rc == 0 and out.count("check: 0 errors found") == 2


def test_storage_needs_the_wave_form():
    rc, out, err = run(CLI, "--storage", "f16")
    assert rc == 2 and "--storage f16 needs --wave" in err
    rc, out, err = run(CLI, "--wave", "--storage", "int8")
    assert rc == 2 and "--storage must be" in err


@pytest.mark.gpu
@pytest.mark.parametrize("extra", [["--storage", "f16"], ["--storage", "f16_hilo"],
                                   ["--storage", "f16_hl"], ["--storage", "bf16", "--kernel", "mma"],
                                   ["--storage", "f16", "--kernel", "tma"],
                                   ["--stencil", "7", "--temporal-block", "4"]])
def test_wave_forms_through_the_driver(extra):
    args = ["--xs", "40", "--ys", "40", "--zs", "128", "--iter", "8", "--wave", "--dt", "0.0005"]
    if "--stencil" not in extra:
        args += ["--stencil", "25"]
    rc, out, err = run(CLI, *(args + extra))
    assert rc == 0, err
    assert "leapfrog wave" in out and "finish compute in" in out
