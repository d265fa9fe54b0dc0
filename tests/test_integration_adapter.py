"""The C++ adapter that INTEGRATION.md gives a maintainer (the reference-side
binding of include/mcacg.h) compiles against the header, links against the
library and runs: on a machine without a GPU its constructor reports the
library's "no CUDA device" error through the adapter's exception; with a GPU
it drives a few steps of the reference's per-step interface."""
import re
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

MAIN = r"""
#include <cmath>
#include <cstdio>
#include "adapter.hpp"
int main(int argc, char **argv) {
    try {
        mcac::GpuAggregatList aggregates(argv[1]);
        aggregates.sort_time_steps(1.0);
        const size_t label = aggregates.pick_random();
        const double dt = aggregates.get_time_step(1.0);
        const std::array<double, 3> dir{1.0, 0.0, 0.0};
        const mcacg_contact c = aggregates.distance_to_next_contact(label, dir, 1e-7);
        const double move = c.distance <= 1e-7 ? c.distance : 1e-7;
        aggregates.translate(label, {move, 0.0, 0.0});
        aggregates.time_forward(label, dt);
        if (c.distance <= 1e-7 && aggregates.merge(c)) aggregates.refresh();
        std::printf("ok %zu %d\n", label, int(std::isfinite(dt)));
    } catch (const std::exception &e) {
        std::printf("error: %s\n", e.what());
    }
    return 0;
}
"""

INI = """[monomers]
number = 200
mean_diameter = 30
dispersion_diameter = 1.25
initialisation_mode = normal
[environment]
volume_fraction = 5e-3
temperature = 1700
[numerics]
random_seed = 3
with_domain_duplication = false
"""


def adapter_source() -> str:
    text = (ROOT / "INTEGRATION.md").read_text()
    section = text[text.index("## C++ adapter"):]
    m = re.search(r"```cpp\n(.*?)```", section, re.S)
    assert m, "no C++ block in the adapter section"
    return m.group(1)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integration_adapter_builds_and_runs(tmp_path, built_library):
    (tmp_path / "adapter.hpp").write_text(adapter_source())
    (tmp_path / "main.cpp").write_text(MAIN)
    (tmp_path / "params.ini").write_text(INI)
    exe = tmp_path / "adapter_main"
    lib_dir = Path(built_library).parent
    cmd = ["g++", "-std=c++17", "-Wall", "-Werror", "-Wno-unused-result", f"-I{ROOT / 'include'}",
           str(tmp_path / "main.cpp"), "-o", str(exe), f"-L{lib_dir}", "-lmcacg", f"-Wl,-rpath,{lib_dir}"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr
    run = subprocess.run([str(exe), str(tmp_path / "params.ini")], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    out = run.stdout.strip()
    sys.path.insert(0, str(ROOT))
    from mcac_gb300 import device_count
    if device_count() > 0:
        assert out.startswith("ok "), out
    else:
        assert out.startswith("error: ") and "device" in out.lower(), out
