"""The header-only C++ layer (include/aperture/scene_renderer.hpp) compiles
against the C ABI, links the library, and reports a missing GPU as an
exception rather than a crash."""
import shutil
import subprocess

import pytest

from conftest import ROOT

PROGRAM = r"""
#include "aperture/scene_renderer.hpp"
#include <cstdio>
int main() {
    using namespace aperture;
    std::vector<SceneObject> objs;
    objs.push_back(SceneObject({0, -0.5f, 0}, {0.5f, 0.01f, 0.5f}, Material::CreateDiffusePureColor({0.7f, 0.7f, 0.7f}), {0, 0, 0}));
    objs.push_back(SceneObject({0, 0.49f, 0}, {0.1f, 0.005f, 0.1f}, Material::CreateLight({17, 12, 4}), {0, 0, 0}));
    objs.push_back(SceneObject::Triangle({-1, -1, -1}, {1, -1, -1}, {0, 1, -1}, Material::CreateGGXPureColor({0.5f, 0.5f, 0.5f}, 0.3f, 0.0f, 0.5f)));
    try {
        SceneRenderer r(objs);
        r.fov_deg = 40.0f;
        std::vector<float3> img = r.Render({8, 8}, {0, 0, 0.45f}, {0, 0, -1}, 2);
        std::printf("rendered %zu %g\n", img.size(), (double)img[27].y);
    } catch (const Error& e) {
        std::printf("error %d %s\n", e.code, e.what());
    }
    return 0;
}
"""


def test_cpp_layer_compiles_links_and_runs(tmp_path):
    import torch
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "app.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "app"
    lib_dir = ROOT / "aperturerendererv3_gb300"
    subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-I", str(ROOT / "include"), "-I",
                    str(ROOT / "include" / "aperture"), "-L", str(lib_dir), "-laperture_gb300",
                    f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    if torch.cuda.is_available():
        assert out.startswith("rendered 64"), out
    else:
        assert out.startswith("error -2"), out
