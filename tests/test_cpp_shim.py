"""The header-only C++ layer (include/aperture/scene_renderer.hpp) compiles
against the C ABI, links the library, and reports a missing GPU as an
exception rather than a crash.  On a GPU, a scene with a textured mesh, the
SDF union and a medium rendered through the C++ layer equals the same scene
rendered through the Python layer bit for bit, and RenderToFile's BMP and PFM
equal the Python writers' files."""
import shutil
import subprocess

import numpy as np
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


FULL_PROGRAM = r"""
#include "aperture/scene_renderer.hpp"
#include <cstdio>
int main(int argc, char** argv) {
    using namespace aperture;
    std::vector<SceneObject> objs;
    objs.push_back(SceneObject({0, 0.49f, 0}, {0.1f, 0.005f, 0.1f}, Material::CreateLight({17, 12, 4}), {0, 0, 0}));
    std::vector<float3> v = {{-0.5f, -0.5f, -0.5f}, {0.5f, -0.5f, -0.5f}, {0.5f, -0.5f, 0.5f}, {-0.5f, -0.5f, 0.5f},
                             {-0.5f, 0.5f, -0.5f}, {0.5f, 0.5f, -0.5f}};
    std::vector<uint32_t> idx = {0, 1, 2, 0, 2, 3, 0, 1, 5, 0, 5, 4};
    Material tex = Material::CreateDiffuseTextured(0);
    Material ggx = Material::CreateGGXPureColor({0.6f, 0.5f, 0.4f}, 0.3f, 0.0f, 0.5f);
    std::vector<float> uv = {0, 0, 1, 0, 1, 1, 0, 0, 1, 1, 0, 1, 0, 0, 1, 0, 1, 1, 0, 0, 1, 1, 0, 1};
    std::vector<float> texels(4 * 4 * 3);
    for (size_t i = 0; i < texels.size(); ++i) texels[i] = 0.2f + 0.6f * (float)((i * 7) % 11) / 10.0f;
    std::vector<float> prims = {AR_SDF_SPHERE, 0.1f, -0.3f, 0.0f, 0.12f, 0, 0, 0,
                                AR_SDF_BOX, -0.1f, -0.35f, -0.1f, 0.1f, 0.1f, 0.08f, 0};
    try {
        SceneRenderer r(objs);
        r.fov_deg = 40.0f;
        r.max_depth = 8;
        r.SetMesh(v, idx, {tex, tex, ggx, ggx});
        r.SetMeshUV(uv);
        r.SetTextures({texels}, {{4, 4}});
        r.SetSdfUnion(prims, 0.05f, Material::CreateDiffusePureColor({0.3f, 0.6f, 0.8f}));
        r.SetMedium({-0.5f, -0.5f, -0.5f}, {0.5f, 0.0f, 0.5f}, 1.0f, 0.8f, 0.2f, 0.05f);
        int diamond = r.AddVolumeToCacheManager({16, 16, 16}, {0, 0, 0}, {1, 1, 1}, AR_SDF_FN_DIAMOND, sdf::CreateDiamond());
        (void)diamond;
        Camera cam(r, "cpp", 24, 16, {0, 0, 1.4f}, {0, 0, -1});
        std::vector<double> xyz = cam.RenderToFile(std::string(argv[1]) + "/img.bmp", 4, AR_TONE_ACES, 1.5f);
        cam.RenderToFile(std::string(argv[1]) + "/img.pfm", 4);
        FILE* f = std::fopen((std::string(argv[1]) + "/xyz.bin").c_str(), "wb");
        std::fwrite(xyz.data(), sizeof(double), xyz.size(), f);
        std::fclose(f);
        std::printf("texels %lld\n", (long long)r.TexelCount());
        // the denoised image, the GPU-built BVH (same hits), a refit of the moved mesh
        auto dump = [&](const char* name, const std::vector<double>& d) {
            FILE* g = std::fopen((std::string(argv[1]) + "/" + name).c_str(), "wb");
            std::fwrite(d.data(), sizeof(double), d.size(), g);
            std::fclose(g);
        };
        r.denoise = true;
        dump("xyz_dn.bin", r.RenderXYZ({24, 16}, {0, 0, 1.4f}, {0, 0, -1}, 4));
        r.denoise = false;
        r.SetBuildMode(AR_BUILD_GPU);
        std::printf("gpu_build_same %d\n", (int)(r.RenderXYZ({24, 16}, {0, 0, 1.4f}, {0, 0, -1}, 4) == xyz));
        std::printf("build_ms_positive %d\n", (int)(r.BuildTimeMs() > 0.0));
        std::vector<float3> moved = v;
        for (float3& p : moved) p.y += 0.05f;
        r.RefitMesh(moved);
        dump("xyz_refit.bin", r.RenderXYZ({24, 16}, {0, 0, 1.4f}, {0, 0, -1}, 4));
    } catch (const Error& e) {
        std::printf("error %d %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
"""


def compile_program(tmp_path, text):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "app.cpp"
    src.write_text(text)
    exe = tmp_path / "app"
    lib_dir = ROOT / "aperturerendererv3_gb300"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", str(src), "-I", str(ROOT / "include"), "-I",
                    str(ROOT / "include" / "aperture"), "-L", str(lib_dir), "-laperture_gb300",
                    f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    return exe


def test_full_cpp_layer_compiles(tmp_path):
    compile_program(tmp_path, FULL_PROGRAM)


@pytest.mark.gpu
def test_cpp_layer_equals_python_layer(tmp_path, cuda_device):
    from aperturerendererv3_gb300 import SceneRenderer
    from aperturerendererv3_gb300._lib import OBJECT_CUBE, SDF_BOX, SDF_SPHERE
    from aperturerendererv3_gb300.scene import Material, Medium, SceneObject, SdfUnion, TriangleMesh, write_bmp, \
        write_pfm
    exe = compile_program(tmp_path, FULL_PROGRAM)
    out = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, check=True).stdout
    assert out.startswith("texels 48"), out   # floats: 16 texels x RGB
    light = SceneObject((0, 0.49, 0), (0.1, 0.005, 0.1), Material.CreateLight((17, 12, 4)), (0, 0, 0), OBJECT_CUBE)
    v = np.array([[-0.5, -0.5, -0.5], [0.5, -0.5, -0.5], [0.5, -0.5, 0.5], [-0.5, -0.5, 0.5], [-0.5, 0.5, -0.5],
                  [0.5, 0.5, -0.5]], np.float32)
    tex, ggx = Material.CreateDiffuseTextured(0), Material.CreateGGXPureColor((0.6, 0.5, 0.4), 0.3, 0.0, 0.5)
    uv = np.array([0, 0, 1, 0, 1, 1, 0, 0, 1, 1, 0, 1] * 2, np.float32).reshape(4, 6)
    mesh = TriangleMesh(v, np.array([[0, 1, 2], [0, 2, 3], [0, 1, 5], [0, 5, 4]], np.uint32),
                        np.array([0, 0, 1, 1], np.int32), [tex, ggx], uv=uv)
    texels = np.array([0.2 + 0.6 * ((i * 7) % 11) / 10.0 for i in range(48)], np.float32).reshape(4, 4, 3)
    sdf = SdfUnion([(SDF_SPHERE, (0.1, -0.3, 0.0), (0.12, 0, 0)), (SDF_BOX, (-0.1, -0.35, -0.1), (0.1, 0.1, 0.08))],
                   0.05, Material.CreateDiffusePureColor((0.3, 0.6, 0.8)))
    med = Medium((-0.5, -0.5, -0.5), (0.5, 0.0, 0.5), sigma_t=1.0, albedo=0.8, g=0.2, emission=0.05)
    r = SceneRenderer([light], mesh=mesh, textures=[texels], sdf=sdf, medium=med)
    img = r.Render((24, 16), (0, 0, 1.4), (0, 0, -1), 4, fov=40.0, max_depth=8)
    cpp = np.fromfile(tmp_path / "xyz.bin", np.float64).reshape(img.shape)
    assert np.array_equal(cpp, img)
    write_bmp(str(tmp_path / "py.bmp"), r.tonemap(img, 1.5, "aces"))
    assert (tmp_path / "py.bmp").read_bytes() == (tmp_path / "img.bmp").read_bytes()
    write_pfm(str(tmp_path / "py.pfm"), img)
    assert (tmp_path / "py.pfm").read_bytes() == (tmp_path / "img.pfm").read_bytes()
    # denoiser, GPU build and refit through the C++ layer
    assert "gpu_build_same 1" in out and "build_ms_positive 1" in out, out
    den = r.Render((24, 16), (0, 0, 1.4), (0, 0, -1), 4, fov=40.0, max_depth=8, denoise=True)
    assert np.array_equal(np.fromfile(tmp_path / "xyz_dn.bin", np.float64).reshape(den.shape), den)
    moved = v.copy()
    moved[:, 1] += np.float32(0.05)
    r.refit_mesh(moved)
    ref = r.Render((24, 16), (0, 0, 1.4), (0, 0, -1), 4, fov=40.0, max_depth=8)
    assert np.array_equal(np.fromfile(tmp_path / "xyz_refit.bin", np.float64).reshape(ref.shape), ref)


def test_cpp_layer_compiles_links_and_runs(tmp_path):
    import torch
    exe = compile_program(tmp_path, PROGRAM)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    if torch.cuda.is_available():
        assert out.startswith("rendered 64"), out
    else:
        assert out.startswith("error -2"), out
