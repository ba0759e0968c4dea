"""The C++ host API (dataBase / solverBase, core/dataBase.h and
core/solverBase.h in the reference): case drivers written for the reference
compile unchanged against dem-sphsource_gb300/host and link
libdemsph_gb300.so; the point generators give the reference's points in the
reference's order; and on a GPU a driver's frames are the same whether
solverBase batches the steps between frames or calls the step functions one
by one."""
import glob
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "dem-sphsource_gb300")
HOST = os.path.join(PKG, "host")
REF = os.environ.get("REF") or os.path.join(os.path.dirname(ROOT), "reference")
DRIVER = os.path.join(ROOT, "tests", "drivers", "tinyDamBreak.cpp")


def cuda_include():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "include", "vector_types.h")):
            return os.path.join(c, "include")
    pytest.skip("CUDA headers not found")


def compile_driver(src, out, ds):
    ds.load_library()  # the library must exist to link against
    cmd = ["g++", "-std=c++17", "-O1", f"-I{cuda_include()}", f"-I{HOST}", f"-I{os.path.join(ROOT, 'include')}",
           src, f"-L{PKG}", "-ldemsph_gb300", f"-Wl,-rpath,{PKG}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_reference_damBreak_driver_compiles_unchanged(ds, tmp_path):
    src = os.path.join(REF, "driver", "cases", "damBreak.cpp")
    if not os.path.exists(src):
        pytest.skip("reference sources not present")
    compile_driver(src, str(tmp_path / "damBreak"), ds)


def test_own_driver_compiles(ds, tmp_path):
    compile_driver(DRIVER, str(tmp_path / "tinyDamBreak"), ds)


POINTS_MAIN = r"""
#include <cstdio>
#include "generatePoints.h"
int main() {
    const double3 o[3] = {{-0.075, -0.075, -0.075}, {0.0, 0.0, 0.0}, {5.2, 0.275, 0.0}};
    const double3 s[3] = {{8.15, 0.85, 0.95}, {0.4, 0.4, 0.3}, {0.15, 0.15, 0.15}};
    const double h[3] = {0.025, 0.01, 0.025};
    for (int k = 0; k < 3; ++k) {
        for (const auto& p : getRegularPackedPoints(o[k], s[k], h[k])) std::printf("%a %a %a\n", p.x, p.y, p.z);
        for (const auto& p : getHexagonalClosePackedPoints(o[k], s[k], h[k])) std::printf("%a %a %a\n", p.x, p.y, p.z);
    }
    std::printf("%a\n", getRegularPackedPoints({0, 0, 0}, {0.001, 1, 1}, 0.01)[0].x);
    return 0;
}
"""


def test_point_generators_match_the_reference(tmp_path):
    ref_hdr = os.path.join(REF, "core", "generatePoints.h")
    if not os.path.exists(ref_hdr):
        pytest.skip("reference sources not present")
    (tmp_path / "main.cpp").write_text(POINTS_MAIN)
    outs = []
    for inc in (HOST, os.path.join(REF, "core")):
        exe = str(tmp_path / f"pts{len(outs)}")
        cmd = ["g++", "-std=c++17", "-O0", f"-I{cuda_include()}", f"-I{inc}", str(tmp_path / "main.cpp"), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        outs.append(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    assert outs[0].count("\n") > 100000
    assert outs[0] == outs[1]


def read_vtu(path):
    text = open(path).read()
    arrays = {}
    for m in re.finditer(r'<DataArray([^>]*)>([^<]*)</DataArray>', text):
        name = re.search(r'Name="([^"]+)"', m.group(1))
        arrays[name.group(1) if name else "Points"] = np.array(m.group(2).split(), dtype=float)
    return arrays


@pytest.mark.gpu
def test_driver_frames_batched_equal_staged(ds, tmp_path):
    exe = str(tmp_path / "tinyDamBreak")
    compile_driver(DRIVER, exe, ds)
    for mode in ("batched", "staged"):
        r = subprocess.run([exe, mode] + (["staged"] if mode == "staged" else []), cwd=tmp_path,
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "Initialization completed." in r.stdout
        assert r.stdout.count("Frame ") == 4, r.stdout
    for kind in ("fluid", "solid"):
        a = sorted(glob.glob(str(tmp_path / "batchedOutput" / f"{kind}_*.vtu")))
        b = sorted(glob.glob(str(tmp_path / "stagedOutput" / f"{kind}_*.vtu")))
        assert [os.path.basename(x) for x in a] == [f"{kind}_{i:04d}.vtu" for i in range(5)]
        assert [os.path.basename(x) for x in b] == [os.path.basename(x) for x in a]
        for fa, fb in zip(a, b):
            assert open(fa).read() == open(fb).read(), fa
    out = tmp_path / "batchedOutput"
    first, last = read_vtu(out / "fluid_0000.vtu"), read_vtu(out / "fluid_0004.vtu")
    assert np.all(np.isfinite(last["Points"]))
    # the column has started to fall: its mean height has gone down
    assert last["Points"][2::3].mean() < first["Points"][2::3].mean()


@pytest.mark.gpu
def test_driver_binary_frames_equal_the_ascii_ones(ds, tmp_path):
    """setBinaryOutput(true): the frames are written as binary VTU by the
    background writer; read back, every array equals the ASCII frame's
    (which prints the FP64 value with ten decimals into a Float32 array)."""
    from vtu import read_vtu as read_any
    exe = str(tmp_path / "tinyDamBreak")
    compile_driver(DRIVER, exe, ds)
    for mode in ("ascii", "bin"):
        r = subprocess.run([exe, mode] + (["binary"] if mode == "bin" else []), cwd=tmp_path, capture_output=True,
                           text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
    for kind in ("fluid", "solid"):
        for i in range(5):
            a = read_any(tmp_path / "asciiOutput" / f"{kind}_{i:04d}.vtu")
            b = read_any(tmp_path / "binOutput" / f"{kind}_{i:04d}.vtu")
            assert 'format="appended"' in b["_header"]
            assert a["STEP"] == b["STEP"]
            for k, v in a.items():
                if k.startswith("_") or k in ("TIME", "STEP"):
                    continue
                assert v.shape == b[k].shape, (kind, i, k)
                if v.dtype.kind == "f":
                    # the decimal text rounds once more than the binary value
                    np.testing.assert_allclose(b[k], v, rtol=2e-7, atol=1e-9, err_msg=f"{kind} {i} {k}")
                else:
                    assert np.array_equal(b[k], v), (kind, i, k)


@pytest.mark.gpu
def test_driver_adds_particles_while_running(ds, tmp_path):
    """addFluid and addCluster at frame 2 of a running driver: the later frames
    hold the new particles (the frame writer follows the larger engine), and
    the run stays finite."""
    from vtu import read_vtu as read_any
    exe = str(tmp_path / "tinyDamBreak")
    compile_driver(DRIVER, exe, ds)
    for mode in ("add", "addbin"):
        r = subprocess.run([exe, mode, "append"] + (["binary"] if mode == "addbin" else []), cwd=tmp_path,
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        out = tmp_path / f"{mode}Output"
        n = [read_any(out / f"fluid_{i:04d}.vtu")["Points"].shape[0] for i in range(5)]
        m = [read_any(out / f"solid_{i:04d}.vtu")["Points"].shape[0] for i in range(5)]
        assert n[0] == n[1] == n[2] < n[3] == n[4] and n[3] - n[2] == 27
        assert m[0] == m[1] == m[2] < m[3] == m[4] and m[3] - m[2] == 8
        last = read_any(out / "fluid_0004.vtu")
        assert np.isfinite(last["Points"]).all() and np.isfinite(last["velocity"]).all()
