"""The C-ABI libraries load and export every symbol their headers declare
(no device compute here)."""

import ctypes
import os
import re

import pytest

from taurus_vap_gb300 import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tv[as]p?_[a-z0-9_]+)\s*\(", text)))


def test_gpu_library_exports_header():
    path = _build.build_gpu()
    L = ctypes.CDLL(path)
    names = declared("tvap.h")
    assert "tvap_calculate_fields" in names and "tvap_project" in names
    for name in names:
        assert hasattr(L, name), name


def test_setup_library_exports_header():
    L = ctypes.CDLL(_build.build_setup())
    for name in declared("tvap_setup.h"):
        assert hasattr(L, name), name


def test_every_status_code_has_a_message():
    """The binding names every status code the header declares."""
    from taurus_vap_gb300 import native

    text = open(os.path.join(ROOT, "include", "tvap.h")).read()
    codes = {int(v) for v in re.findall(r"\bTVAP_ERR_[A-Z0-9_]+\s*=\s*(\d+)", text)}
    assert codes and 19 in codes
    assert codes <= set(native.ERRORS), sorted(codes - set(native.ERRORS))
    err = native.TvapError(19, "tvap_project", "detail")
    assert err.code == 19 and "bounded wait" in str(err) and "detail" in str(err)


def test_missing_library_raises(monkeypatch, tmp_path):
    """No CPU fallback: without the built device library the binding raises."""
    from taurus_vap_gb300 import native

    monkeypatch.setattr(native._build, "GPU_LIB", str(tmp_path / "libtvap_gpu.so"))
    monkeypatch.setattr(native, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        native.lib()


def test_context_without_a_device_raises():
    """Without a CUDA device, creating a context is a CUDA status error, not
    a silent fallback."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from taurus_vap_gb300 import model as M
    from taurus_vap_gb300 import native

    _build.build_gpu()
    mdl = M.sd_model(seed=1)
    with pytest.raises(native.TvapError) as e:
        native.Context(mdl.basis, mdl.ham, device=0)
    assert e.value.code == 2


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes structures of the binding have the sizes and field offsets
    of the header's tvap_pnp, tvap_pnp_obs and tvap_proj_opts (compiled with
    the host C compiler)."""
    import shutil
    import subprocess

    from taurus_vap_gb300 import native

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pnp = [f[0] for f in native.TvapPnp._fields_]
    opts = [f[0] for f in native.TvapProjOpts._fields_]
    obs = [f[0] for f in native.TvapPnpObs._fields_]
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "tvap.h"', "int main(void) {"]
    lines.append('  printf("pnp %zu\\n", sizeof(tvap_pnp));')
    lines += [f'  printf("pnp.{k} %zu\\n", offsetof(tvap_pnp, {k}));' for k in pnp]
    lines.append('  printf("opts %zu\\n", sizeof(tvap_proj_opts));')
    lines += [f'  printf("opts.{k} %zu\\n", offsetof(tvap_proj_opts, {k}));' for k in opts]
    lines.append('  printf("obs %zu\\n", sizeof(tvap_pnp_obs));')
    lines += [f'  printf("obs.{k} %zu\\n", offsetof(tvap_pnp_obs, {k}));' for k in obs]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    assert int(got["pnp"]) == ctypes.sizeof(native.TvapPnp)
    assert int(got["opts"]) == ctypes.sizeof(native.TvapProjOpts)
    for k in pnp:
        assert int(got[f"pnp.{k}"]) == getattr(native.TvapPnp, k).offset, k
    for k in opts:
        assert int(got[f"opts.{k}"]) == getattr(native.TvapProjOpts, k).offset, k
    assert int(got["obs"]) == ctypes.sizeof(native.TvapPnpObs)
    for k in obs:
        assert int(got[f"obs.{k}"]) == getattr(native.TvapPnpObs, k).offset, k


def test_option_numbers_match_the_header():
    # the binding's OPT_* constants are the header's TVAP_OPT_* enumerators
    from taurus_vap_gb300.native import Context

    text = open(os.path.join(ROOT, "include", "tvap.h")).read()
    enum = dict((m.group(1), int(m.group(2))) for m in re.finditer(r"TVAP_OPT_([A-Z_]+)\s*=\s*(\d+)", text))
    assert enum, "no TVAP_OPT_* enumerators in tvap.h"
    for name, value in enum.items():
        assert getattr(Context, "OPT_" + name) == value, name
