"""CPU test: the C++ shims in INTEGRATION.md (the code a maintainer of the
reference would add to bind the C ABI) compile against include/gsap.h."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT


def cpp_blocks():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```cpp\n(.*?)```", text, flags=re.S)


def test_integration_shims_compile(tmp_path):
    gxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not gxx or not os.path.exists(os.path.join(cuda_inc, "vector_types.h")):
        pytest.skip("needs g++ and the CUDA headers (float4 / int2 of the reference's code)")
    blocks = cpp_blocks()
    assert len(blocks) >= 4

    def pick(marker):
        found = [b for b in blocks if marker in b]
        assert len(found) == 1, marker
        return found[0]

    shim, demo_step, fused_step = pick("class Sap"), pick("gsap_rb_integrate(rb"), pick("gsap_rb_step(")
    standalone = [b for b in blocks if b not in (shim, demo_step, fused_step)]
    src = "\n".join([
        "#include <vector_types.h>",
        shim,
        *standalone,
        "void demo_step(gsap_rb* rb, Sap& sap, float dt) {",
        demo_step,
        "}",
        "void fused_step(gsap_rb* rb, gsap_sap* sapHandle, float dt, void* stream) {",
        fused_step,
        "}",
    ])
    path = tmp_path / "integration_shims.cpp"
    path.write_text(src)
    p = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"),
                        "-I", cuda_inc, str(path)], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
