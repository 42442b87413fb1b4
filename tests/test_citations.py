"""Every reference citation on the C ABI (include/vlb.h) lands on what it names.

The header names, beside each declaration, the reference interface it
replaces as `path:first-last`.  This test opens the reference checkout
(VLB_REFERENCE_DIR; skipped when it is absent) and checks, for each citation,
that the cited lines exist and contain the symbol or statement the
declaration relies on.  A citation that is not in the table below fails the
test, so a new or moved citation has to be checked here.
"""
import os
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF = os.environ.get("VLB_REFERENCE_DIR")

# citation -> text that must occur inside the cited lines
EXPECT = {
    "src/baker/main.cpp:26-40": "catch",
    "src/application.cpp:265-273": "waitForFences",
    "src/application.cpp:540-556": "Application::Application",
    "src/baker/light_baker.cpp:80-101": "probePositionsFromBoudingBox",
    "src/scene_manager.cpp:1013-1034": "SceneManager::pushScene",
    "src/scene_manager.cpp:339-442": "buildAccelerationStructures",
    "shaders/structures.h:20-26": "struct Vertex",
    "src/scene_manager.cpp:214-217": "getBounds",
    "shaders/env_map.rgen:18-28": "toVector(x2phi",
    "shaders/sh.comp:27-41": "pixelArea",
    "src/skybox_manager.cpp:284-298": "SkyboxManager::pushSkybox",
    "src/skybox_manager.cpp:107-130": "Skybox_t::computeSH",
    "shaders/skybox_sh.comp:27-39": "PI / 2.0f",
    "shaders/sh.comp:27-39": "sin(theta)",
    "src/skybox_manager.cpp:18": "STBI_rgb_alpha",
    "src/application.cpp:690": "eB8G8R8A8Unorm",
    "shaders/main.rmiss:37-41": "texture(skybox",
    "src/baker/light_baker.cpp:287-328": "LightBaker::bake",
    "src/baker/env_map_generator.cpp:325-359": "EnvMapGenerator::getMap",
    "src/baker/light_baker.cpp:294-322": "lmax * sizeof(glm::vec3)",
    "shaders/env_map.rgen:22-23": "tmax",
    "shaders/env_map.rchit:81": "shadowBias = 0.005f",
    "src/baker/light_baker.cpp:20-74": "LightBaker::LightBaker",
    "src/baker/main.cpp:22-24": "baker.bake()",
    "shaders/sh.comp:23-42": "coeffs[l * (l + 1) + m]",
    "shaders/sh_sum.comp:35-52": "1250.0f",
    "src/baker/light_baker.cpp:375-401": "LightBaker::serialize",
    "src/scene_manager.cpp:613-648": "loadBakedLight",
    "src/scene_manager.cpp:257-337": "fetchVertices",
    "shaders/main.rchit:124-168": "gridVertices",
    "shaders/sh.rmiss:23-39": "shOffset",
    "shaders/skybox_sh.rmiss:14-25": "skyboxRadiance",
    "src/baker/env_map_generator.hpp:39": "eR8G8B8A8Unorm",
    "src/baker/light_baker.cpp:306-307": "saveImage",
    "src/baker/env_map_generator.cpp:73-112": "EnvMapGenerator::saveImage",
    "shaders/env_map.rchit:101": "sRGB(",
    "shaders/main.rmiss:40": "sRGB(",
    "shaders/main.rchit:49-56": "vec3 sRGB",
    "shaders/sh_sum.comp:51": "1250.0f",
    "shaders/env_map.rchit:51-102": "traceRayEXT",
    "shaders/shadow.rmiss:6-9": "inShadow = false",
    "src/baker/light_baker.cpp:110-121": "SHCoeffs = createBuffer",
    "src/baker/light_baker.cpp:298-322": "memcpy(ptr, dataPtr",
}

CITE = re.compile(r"((?:src|shaders)/[A-Za-z_/]+\.(?:cpp|hpp|h|comp|rgen|rchit|rmiss)):(\d+)(?:-(\d+))?"
                  r"((?:, :\d+(?:-\d+)?)*)")


def citations(text: str):
    """(path, first, last) for every citation, including `, :a-b` continuations."""
    out = []
    for m in CITE.finditer(text):
        path = m.group(1)
        out.append((path, int(m.group(2)), int(m.group(3) or m.group(2))))
        for c in re.finditer(r":(\d+)(?:-(\d+))?", m.group(4) or ""):
            out.append((path, int(c.group(1)), int(c.group(2) or c.group(1))))
    return out


def key(path, a, b):
    return f"{path}:{a}" if a == b else f"{path}:{a}-{b}"


def test_header_citations_are_listed():
    """Runs without the checkout: every citation of the header has an entry."""
    text = (ROOT / "include" / "vlb.h").read_text()
    missing = sorted({key(*c) for c in citations(text)} - set(EXPECT))
    assert not missing, f"citations without an expectation: {missing}"


@pytest.mark.skipif(not REF or not Path(REF).is_dir(), reason="reference checkout absent (set VLB_REFERENCE_DIR)")
def test_header_citations_land_on_their_symbols():
    text = (ROOT / "include" / "vlb.h").read_text()
    bad = []
    for path, a, b in citations(text):
        lines = (Path(REF) / path).read_text(errors="replace").splitlines()
        if not (1 <= a <= b <= len(lines)):
            bad.append((key(path, a, b), f"outside the file ({len(lines)} lines)"))
            continue
        body = "\n".join(lines[a - 1:b])
        want = EXPECT[key(path, a, b)]
        if want not in body:
            bad.append((key(path, a, b), f"no {want!r}"))
    assert not bad, bad
