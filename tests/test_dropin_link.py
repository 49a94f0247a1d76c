"""Source-level drop-in: the reference's own BarnesHutParticleSystem.cpp and
debug.cpp compile against include/Particle_cuda.cuh and link against
libstellar_bh.so (its nine wrapper calls resolve to this library).

CPU only; runs when the STELLARSOLVER_REF environment variable names the
reference sources, skipped otherwise."""
import os
import shutil
import subprocess

import pytest

REF = os.environ.get("STELLARSOLVER_REF", "")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(not REF or not os.path.isfile(os.path.join(REF, "BarnesHutParticleSystem.cpp")),
                    reason="STELLARSOLVER_REF does not name the reference sources")
def test_reference_host_class_links_against_library(tmp_path):
    from stellarsolver_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    nvcc = build.nvcc()
    main = tmp_path / "main.cpp"
    main.write_text(
        '#include "BarnesHutParticleSystem.h"\n'
        "int main(int argc, char**) {\n"
        "  if (argc > 5) { SimulationParameters p{}; BarnesHutParticleSystem s(p, 1024);\n"
        "    s.reset(); s.update(); return s.getNumParticles(); }\n"
        "  return 0; }\n")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + REF]
    objs = []
    for src in (os.path.join(REF, "BarnesHutParticleSystem.cpp"), os.path.join(REF, "debug.cpp"),
                str(main)):
        obj = tmp_path / (os.path.basename(src) + ".o")
        subprocess.run([nvcc, "-std=c++11", "-x", "cu", "-w"] + inc + ["-c", src, "-o", str(obj)],
                       check=True, capture_output=True)
        objs.append(str(obj))
    exe = tmp_path / "app"
    r = subprocess.run([nvcc, "-o", str(exe)] + objs +
                       ["-L" + build.LIB_DIR, "-lstellar_bh", "-Xlinker", "-rpath=" + build.LIB_DIR],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert shutil.which("nm") is None or b"ResetArrays" in subprocess.run(
        ["nm", "-D", build.LIB], capture_output=True).stdout
