"""CPU checks of the drop-in boundary: the library builds, loads and exports
every entry point declared in include/qbgpu.h (no compute without a GPU)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    txt = (ROOT / "include" / "qbgpu.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:qbg_status|size_t)\s+(qbg_\w+)\s*\(", txt, flags=re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("qbg_geom_create", "qbg_assemble", "qbg_beyn_create", "qbg_beyn_moments", "qbg_sigma_min"):
        assert s in syms


def test_library_exports_every_declared_symbol(qb):
    from qbgpu import _lib
    lib = _lib.load()
    for s in declared_symbols():
        assert hasattr(lib, s), s
    # the ctypes signature table covers the whole header
    assert sorted(_lib.exported_symbols()) == declared_symbols()


def test_error_path_without_gpu_work(qb):
    """Invalid arguments are rejected before any device call."""
    from qbgpu import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    st = lib.qbg_geom_create(None, ctypes.byref(h))
    assert st == _lib.QBG_EINVAL
    assert "null" in _lib.last_error()
    st = lib.qbg_beyn_moments(None, None, 0, None, None, None)
    assert st == _lib.QBG_EINVAL


def test_ebim_argument_checks_without_gpu_work(qb):
    """qbg_ebim_eig / qbg_ebim_solve reject bad sizes, windows and outputs
    before any device call."""
    from qbgpu import _lib
    lib = _lib.load()
    cnt = ctypes.c_int32()
    out = (ctypes.c_double * 16)()
    tens = (ctypes.c_double * 8)()
    buf = (ctypes.c_double * 8)()
    args = (12.0, 0.1, 4, 0, 8, out, tens, ctypes.byref(cnt), None)
    assert lib.qbg_ebim_eig(0, buf, buf, buf, *args) == _lib.QBG_EINVAL            # n < 1
    assert lib.qbg_ebim_eig(2, None, buf, buf, *args) == _lib.QBG_EINVAL           # missing A
    assert lib.qbg_ebim_eig(2, buf, buf, buf, 12.0, 0.0, 4, 0, 8, out, tens, ctypes.byref(cnt), None) \
        == _lib.QBG_EINVAL                                                          # dk <= 0
    assert lib.qbg_ebim_eig(2, buf, buf, buf, 12.0, 0.1, 0, 0, 8, out, tens, ctypes.byref(cnt), None) \
        == _lib.QBG_EINVAL                                                          # nev < 1
    assert lib.qbg_ebim_eig(2, buf, buf, buf, 12.0, 0.1, 4, 0, 8, None, tens, ctypes.byref(cnt), None) \
        == _lib.QBG_EINVAL                                                          # cap > 0 without outputs
    assert lib.qbg_ebim_solve(None, *args) == _lib.QBG_EINVAL                      # no geometry
