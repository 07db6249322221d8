"""The drop-in shims of dials-metal_gb300/shim/ compiled against the
reference's own headers, where the reference tree is present (this test is
skipped elsewhere): dext_sfgb.cc is linked with the reference's unchanged
policy half (src/spots/dext_gpu.cc) and libsfgb.so into a program that calls
gpu::backend / available / unavailable_reason / find<T> as find_spots.cc does;
the labeller, refl and decompress shims compile against dials_spots.hh,
refl.hh and decompress.hh. Without a device the program checks the refusals
the reference makes before touching one (-1 for a null frame) and that a
device failure throws, as dext_cuda.cu does."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO

REF_SPOTS = os.environ.get("SFGB_REFERENCE_SRC", "/root/reference/src/spots")
SHIM = os.path.join(REPO, "dials-metal_gb300", "shim")
INCLUDE = os.path.join(REPO, "include")

pytestmark = pytest.mark.skipif(
    not os.path.exists(os.path.join(REF_SPOTS, "dext_gpu.hh")) or shutil.which("g++") is None,
    reason="the reference's src/spots headers (or g++) are not here")

DRIVER = r"""
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>
#include "dext_gpu.hh"

int main() {
  std::printf("backend=%s\n", gpu::backend());
  const bool on = gpu::available();
  std::printf("available=%d reason=%s\n", on ? 1 : 0, gpu::unavailable_reason().c_str());
  std::vector<SignalPixel> out(3);
  const int null_rc = gpu::find<std::uint32_t>(nullptr, out, 64, 64);
  std::printf("null_rc=%d null_size=%zu\n", null_rc, out.size());
  std::vector<std::uint32_t> frame(64 * 64, 1u);
  try {
    const int rc = gpu::find<std::uint32_t>(frame.data(), out, 64, 64);
    std::printf("find_rc=%d found=%zu\n", rc, out.size());
  } catch (const std::runtime_error &e) {
    std::printf("threw=%s\n", e.what());
  }
  std::vector<std::uint16_t> frame16(64 * 64, 1u);
  try {
    const int rc = gpu::find<std::uint16_t>(frame16.data(), out, 64, 64);
    std::printf("find16_rc=%d found16=%zu\n", rc, out.size());
  } catch (const std::runtime_error &e) {
    std::printf("threw16=%s\n", e.what());
  }
  return 0;
}
"""


def _lib_dir():
    from sfgb import _paths
    path = _paths.core_lib()
    if not os.path.exists(path):
        pytest.skip("libsfgb.so is not built")
    return os.path.dirname(path)


def _gxx(args, cwd):
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Wextra", *args], cwd=cwd,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def test_dext_shim_links_with_the_reference_policy_half(tmp_path):
    libdir = _lib_dir()
    (tmp_path / "driver.cc").write_text(DRIVER)
    inc = ["-I", REF_SPOTS, "-I", INCLUDE]
    _gxx([*inc, "-o", "driver", "driver.cc", os.path.join(SHIM, "dext_sfgb.cc"),
          os.path.join(REF_SPOTS, "dext_gpu.cc"), "-L", libdir, "-lsfgb",
          f"-Wl,-rpath,{libdir}"], tmp_path)
    r = subprocess.run([str(tmp_path / "driver")], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    text = r.stdout
    assert "backend=CUDA" in text
    # dext.cc:14-23: a null frame is a bad argument, refused before any device
    # work, and the output is cleared.
    assert "null_rc=-1 null_size=0" in text
    if "available=0" in text:
        assert "reason=" in text and "reason=\n" not in text
        # No device: the reference throws "CUDA: ..." (dext_cuda.cu:46-51).
        assert "threw=CUDA: " in text and "threw16=CUDA: " in text, text
    else:
        assert "find_rc=0" in text and "find16_rc=0" in text, text


@pytest.mark.parametrize("unit", ["dials_spots_sfgb.hh", "refl_sfgb.hh"])
def test_labeller_and_refl_shims_compile(tmp_path, unit):
    src = tmp_path / "unit.cc"
    src.write_text(f'#include "{unit}"\nint main() {{ return 0; }}\n')
    _gxx(["-fsyntax-only", "-I", SHIM, "-I", REF_SPOTS, "-I", INCLUDE, str(src)], tmp_path)


def test_decompress_shim_compiles(tmp_path):
    _gxx(["-c", "-I", REF_SPOTS, "-I", INCLUDE, os.path.join(SHIM, "decompress_sfgb.cc"),
          "-o", str(tmp_path / "d.o")], tmp_path)
