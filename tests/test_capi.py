"""CPU checks of the C ABI: the library loads, exports every symbol that
include/*.h declares, and its host-only entry points behave (no GPU calls)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"//.*", "", text)
        for m in re.finditer(r"\b((?:oh|cuda)[A-Za-z0-9_]*)\s*\(", text):
            if not text[:m.start()].rstrip().endswith(("typedef", "#define")):
                names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(lib_built):
    from openholo_gb300 import _lib
    names = declared_functions()
    assert {"oh_depthmap_generate", "cudaFFT", "oh_pointcloud", "oh_fft2d"} <= names
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = sorted(n for n in names if n not in exported)
    assert not missing, missing
    # the ctypes table covers the native API of oh.h
    native = {n for n in names if n.startswith("oh_") and n != "oh_shim_last_status"}
    assert native <= set(_lib.SIGNATURES), sorted(native - set(_lib.SIGNATURES))


def test_host_only_entry_points(lib_built):
    L = lib_built
    assert L.oh_status_string(0) == b"OH_OK"
    assert L.oh_status_string(2) == b"OH_ERR_UNSUPPORTED_SIZE"
    assert b"sm_103a" in L.oh_version()
    assert isinstance(L.oh_kernel_launch_count(), int)


def test_config_parser_sample(lib_built):
    from openholo_gb300 import depthmap as dm
    p = dm.read_config(ROOT / "tests/golden/config_sample.txt")
    assert (p.pnx, p.pny) == (1920, 360)
    assert p.ppx == pytest.approx(12.7e-3 / 1000 / 3, rel=1e-15)
    assert p.ppy == pytest.approx(12.7e-6, rel=1e-15)
    assert p.lambda_ == 633e-9 and p.field_lens == 0.5
    assert (p.near_depthmap, p.far_depthmap) == (0.15, 0.45)    # min/max swap of readConfig
    assert p.num_of_depth == 64 and p.flag_change_depth_quantization == 1
    assert [p.render_depth[i] for i in range(p.n_render_depth)] == [5, 9, 12]
    assert p.transform_viewing_window == 1 and p.pad == 1
    assert (p.rand_phase_re, p.rand_phase_im) == (1.0, 0.0)


def test_config_parser_reference_file(lib_built):
    ref = Path("/root/reference/OpenHolo_DepthMap/bin/config_openholo.txt")
    if not ref.exists():
        pytest.skip("reference tree not present")
    from openholo_gb300 import depthmap as dm
    p = dm.read_config(ref)
    assert (p.pnx, p.pny) == (11520, 2160)
    assert p.ppx == pytest.approx(25.4e-3 / 2250 / 3, rel=1e-15)
    assert p.num_of_depth == 256 and p.n_render_depth == 256
    assert p.near_depthmap == 0.2 and p.far_depthmap == 0.7 and p.lambda_ == 522e-9


def test_config_parser_errors(lib_built, tmp_path):
    from openholo_gb300 import depthmap as dm
    from openholo_gb300._lib import OhError
    with pytest.raises(OhError):
        dm.read_config(tmp_path / "missing.txt")
    bad = (ROOT / "tests/golden/config_sample.txt").read_text().replace("640*3", "640*(3")
    (tmp_path / "bad.txt").write_text(bad)
    with pytest.raises(OhError):
        dm.read_config(tmp_path / "bad.txt")
    trunc = "\n".join((ROOT / "tests/golden/config_sample.txt").read_text().splitlines()[:30])
    (tmp_path / "trunc.txt").write_text(trunc)
    with pytest.raises(OhError):
        dm.read_config(tmp_path / "trunc.txt")


def test_null_arguments_rejected_without_gpu(lib_built):
    from openholo_gb300 import _lib
    L = lib_built
    assert L.oh_depthmap_levels(None, None, None) == 1
    assert L.oh_ctx_create(None, 0) == 1


def test_library_resolves_its_own_symbols(lib_built):
    """Every undefined dynamic symbol of the library comes from the system
    libraries (versioned glibc / libstdc++ / libgcc entries or weak ones): a
    library-internal function declared in the wrong namespace would show up
    here as an unversioned undefined symbol."""
    import shutil
    import subprocess
    if not shutil.which("nm"):
        pytest.skip("nm not available")
    from openholo_gb300 import build as B
    out = subprocess.run(["nm", "-D", "--undefined-only", str(B.LIB)], capture_output=True, text=True).stdout
    bad = [ln for ln in out.splitlines() if ln.split() and ln.split()[0] == "U" and "@" not in ln]
    assert not bad, bad[:10]
