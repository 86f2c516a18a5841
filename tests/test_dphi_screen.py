"""The filter's dphi screen: where it decides without the cut's two atan2,
its decision equals the cut's on seven million triplets, a third of them
built to sit within 1e-4 rad of the cut (tests/c/dphi_screen.c, compiled
with the host build contract of trax_math.h).  The kernels include the same
header; the GPU parity tests check the filter end to end."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dphi_screen_agrees_with_the_cut(tmp_path):
    exe = str(tmp_path / "dphi_screen")
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
                    "-fno-fast-math", "-I" + os.path.join(ROOT, "trax_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "c", "dphi_screen.c"), "-lm", "-o", exe], check=True)
    p = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    cases, undecided, mism, served, served_undecided = (int(v) for v in p.stdout.split()[1::2])
    assert mism == 0
    assert cases > 7_000_000 and undecided > 0
    # random triplets under the cuts the screen serves: nearly all decided
    assert served_undecided < served // 1000, p.stdout
