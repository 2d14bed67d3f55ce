"""The drop-in shim of the repository's integration guide -- mmc_run_cu
implemented over libmmcgb, the guide's C block -- compiles against the reference's own headers
(src/mmc_cu_host.h, mmc_utils.h, mmc_mesh.h), so every mcconfig/tetmesh
field it maps exists with a compatible type.  Needs the reference sources:
their location comes from MMC_REFERENCE or from the reference build in
oracle/_ref (oracle/build_ref.sh records it); without them the test skips."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_src():
    ref = os.environ.get("MMC_REFERENCE")
    rec = os.path.join(ROOT, "oracle", "_ref", "REF_PATH")
    if not ref and os.path.exists(rec):
        ref = open(rec).read().strip()
    if not ref or not os.path.exists(os.path.join(ref, "src", "mmc_cu_host.h")):
        return None
    return os.path.join(ref, "src")


def test_integration_shim_compiles_against_reference_headers(tmp_path):
    src = reference_src()
    if src is None:
        pytest.skip("reference sources not found (set MMC_REFERENCE)")
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = re.search(r"```c\n(.*?)```", doc[doc.index("## Drop-in shim"):], re.S).group(1)
    assert "mmc_run_cu(mcconfig* cfg, tetmesh* mesh, raytracer* tracer)" in block
    assert "c.accumulate = 1" in block
    f = tmp_path / "mmc_run_cu_shim.c"
    f.write_text(block)
    cmd = ["gcc", "-c", "-x", "c", "-std=gnu99", "-Wall", "-Werror", "-I" + src,
           "-I" + os.path.join(src, "zmat", "easylzma"), "-I" + os.path.join(src, "ubj"),
           "-I" + os.path.join(ROOT, "include"), "-DMMC_XORSHIFT",
           "-include", os.path.join(ROOT, "oracle", "ref_shim.h"), str(f), "-o", str(tmp_path / "shim.o")]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert p.returncode == 0, p.stdout
