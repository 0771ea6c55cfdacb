"""The C ABI library without a GPU: it loads, exports every function the
public header declares, its struct layouts match the header as compiled by
a C compiler, and argument validation fails cleanly (these errors are
raised before any CUDA call)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "lettuce_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(lgb_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol(lgb):
    from lettuce_gb300 import _lib
    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 7
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_lib.EXPORTED)
    assert L.lgb_abi_version() == _lib.ABI_VERSION
    assert L.lgb_reduce_scratch_bytes() > 0


def test_struct_layout_matches_header(tmp_path, lgb):
    from lettuce_gb300 import _lib
    src = tmp_path / "probe.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "lettuce_gb300.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\","
        " sizeof(lgb_step_desc),"
        " offsetof(lgb_step_desc, sub), offsetof(lgb_step_desc, options),"
        " sizeof(lgb_substep), offsetof(lgb_substep, rho), offsetof(lgb_substep, u_stride),"
        " offsetof(lgb_step_desc, accel), offsetof(lgb_step_desc, smagorinsky_constant),"
        " offsetof(lgb_step_desc, link_bits), offsetof(lgb_step_desc, force_out));"
        "return 0;}\n")
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    S, D = _lib.Substep, _lib.StepDesc
    assert got == [ctypes.sizeof(D), D.sub.offset, D.options.offset, ctypes.sizeof(S),
                   S.rho.offset, S.u_stride.offset, D.accel.offset,
                   D.smagorinsky_constant.offset, D.link_bits.offset, D.force_out.offset]


def _desc(**kw):
    from lettuce_gb300 import _device, _lib
    d = _device.new_desc(kw.pop("stencil", _lib.D2Q9), kw.pop("storage", _lib.F32),
                         kw.pop("res", [8, 8]))
    d.collision = _lib.BGK
    d.tau = 0.6
    d.f_in = 0x1000
    d.f_out = 0x2000
    for k, v in kw.items():
        setattr(d, k, v)
    return d


@pytest.mark.parametrize("kw,msg", [
    (dict(abi_version=99), "ABI version"),
    (dict(stencil=7), "unknown stencil"),
    (dict(storage=9), "unknown storage"),
    (dict(collision=3, stencil=4, res=[4, 4, 4]), "KBC collision is only defined"),
    (dict(pattern=42), "unknown access pattern"),
    (dict(f_out=0x1000), "distinct input and output"),
    (dict(tau=0.0), "relaxation time must be positive"),
    (dict(res=[0, 8]), "must be positive"),
    (dict(res=[70000, 70000]), "exceeds"),
    (dict(f_in=0), "NULL"),
    (dict(collision=7), "unknown collision"),
    (dict(collision=6), "MRT collision needs its tables"),
    (dict(force=3), "unknown force"),
    (dict(collision=2, tau_minus=1.0, force=1, force_tau=0.8), "needs the BGK or Smagorinsky"),
    (dict(force=1, force_tau=0.0), "force's tau must be positive"),
    (dict(options=4), "unknown option bits"),
])
def test_step_validation_errors(lgb, kw, msg):
    from lettuce_gb300 import _lib
    L = _lib.load()
    d = _desc(**kw)
    rc = L.lgb_step(ctypes.byref(d), None)
    assert rc != 0
    assert msg in L.lgb_last_error().decode()


def test_step_validation_masked(lgb):
    from lettuce_gb300 import _lib
    L = _lib.load()
    d = _desc(flags=0x3000, n_sub=2, collision_index=0)
    d.sub[0].kind = _lib.SUB_COLLISION
    d.sub[1].kind = _lib.SUB_EQUILIBRIUM_PU  # without rho/u
    assert L.lgb_step(ctypes.byref(d), None) != 0
    assert "lacks rho/u" in L.lgb_last_error().decode()
    d = _desc(flags=0x3000, n_sub=3, collision_index=0, no_stream_bits=0x4000,
              pattern=_lib.AA_EVEN)
    d.sub[0].kind = _lib.SUB_COLLISION
    d.sub[1].kind = _lib.SUB_BOUNCE_BACK
    d.sub[2].kind = _lib.SUB_ANTI_BOUNCE_BACK
    d.sub[2].sign = 1
    assert L.lgb_step(ctypes.byref(d), None) != 0
    assert "AA pattern" in L.lgb_last_error().decode()
    d = _desc(flags=0x3000, n_sub=3, collision_index=1)
    d.sub[0].kind = _lib.SUB_BOUNCE_BACK
    d.sub[1].kind = _lib.SUB_BOUNCE_BACK
    assert L.lgb_step(ctypes.byref(d), None) != 0
    assert "collision_index" in L.lgb_last_error().decode()
    # halfway bounce-back links: pulling patterns only, with flags; a force
    # output only with links (all rejected before any device call)
    for kw, msg in [(dict(link_bits=0x5000), "need the flag field"),
                    (dict(flags=0x3000, n_sub=1, collision_index=0, link_bits=0x5000,
                          pattern=_lib.PUSH), "pulling streams"),
                    (dict(flags=0x3000, n_sub=1, collision_index=0, link_bits=0x5000,
                          pattern=_lib.AA_EVEN, f_out=0x1000), "pulling streams"),
                    (dict(force_out=0x6000), "without link_bits"),
                    (dict(force_links=0x6000), "without link_bits"),
                    (dict(flags=0x3000, n_sub=1, collision_index=0, link_bits=0x5000,
                          force_out=0x6000, n_force_links=4), "force links"),
                    (dict(flags=0x3000, n_sub=1, collision_index=0, link_bits=0x5000,
                          force_out=0x6000, force_links=0x7000, n_force_links=4),
                     "force_scratch"),
                    (dict(link_val=0x6000), "without link_bits"),
                    (dict(flags=0x3000, n_sub=1, collision_index=0, link_bits=0x5000,
                          link_val=0x6000, link_base=0x7000, link_pairs=0x8000,
                          n_links=3), "interpolated links need")]:
        d = _desc(**kw)
        d.sub[0].kind = _lib.SUB_COLLISION
        assert L.lgb_step(ctypes.byref(d), None) != 0
        assert msg in L.lgb_last_error().decode()


def test_reduce_and_convert_validation(lgb):
    from lettuce_gb300 import _lib
    L = _lib.load()
    r = _lib.i32x3([8, 8])
    lo = _lib.i32x3([0, 0])
    hi = _lib.i32x3([9, 8])
    rc = L.lgb_reduce(_lib.D2Q9, _lib.F32, ctypes.cast(r, ctypes.c_void_p), 0x1000, 0,
                      ctypes.cast(lo, ctypes.c_void_p), ctypes.cast(hi, ctypes.c_void_p),
                      None, 0x2000, 0x3000, None)
    assert rc != 0 and "box" in L.lgb_last_error().decode()
    assert L.lgb_convert(_lib.D2Q9, 5, 0x1000, _lib.F32, 0x2000, 10, None) != 0
    assert L.lgb_convert(_lib.D2Q9, _lib.F32, 0x1000, _lib.F32, 0x2000, 0, None) == 0


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from lettuce_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "library_path", lambda: str(tmp_path / "nope.so"))
    with pytest.raises(_lib.LibraryError, match="no fallback"):
        _lib.load()


def test_batch_struct_layouts_match_header(tmp_path, lgb):
    """the numpy / ctypes mirrors of the batch tables and descriptor have
    the header's sizes and offsets"""
    from lettuce_gb300._batched import DOMAIN_DTYPE, TILE_DTYPE, BatchDesc
    src = tmp_path / "probe_batch.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "lettuce_gb300.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\","
        " sizeof(lgb_batch_domain), offsetof(lgb_batch_domain, tau),"
        " sizeof(lgb_batch_tile), sizeof(lgb_batch_desc),"
        " offsetof(lgb_batch_desc, domains), offsetof(lgb_batch_desc, f_out),"
        " offsetof(lgb_batch_desc, pool_elements), offsetof(lgb_batch_desc, status),"
        " offsetof(lgb_batch_desc, rates));"
        "return 0;}\n")
    exe = tmp_path / "probe_batch"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == [DOMAIN_DTYPE.itemsize, DOMAIN_DTYPE.fields["tau"][1], TILE_DTYPE.itemsize,
                   ctypes.sizeof(BatchDesc), BatchDesc.domains.offset, BatchDesc.f_out.offset,
                   BatchDesc.pool_elements.offset, BatchDesc.status.offset,
                   BatchDesc.rates.offset]


def test_init_and_enstrophy_validation(lgb):
    """lgb_equilibrium, lgb_init_fneq and lgb_enstrophy refuse bad arguments
    before any device call"""
    from lettuce_gb300 import _lib
    L = _lib.load()
    r2 = _lib.i32x3([8, 6])
    rs = (ctypes.c_int64 * 3)(0, 0, 0)
    us = (ctypes.c_int64 * 4)(0, 0, 0, 0)
    R, RS, US = (ctypes.cast(x, ctypes.c_void_p) for x in (r2, rs, us))
    cases = [
        (lambda: L.lgb_equilibrium(9, _lib.F32, R, 0x1000, RS, 0x2000, US, 0x3000, None, None,
                                   None), "unknown stencil"),
        (lambda: L.lgb_equilibrium(_lib.D2Q9, 7, R, 0x1000, RS, 0x2000, US, 0x3000, None, None,
                                   None), "unknown storage"),
        (lambda: L.lgb_equilibrium(_lib.D2Q9, _lib.F32, R, None, RS, 0x2000, US, 0x3000, None,
                                   None, None), "NULL"),
        (lambda: L.lgb_equilibrium(_lib.D2Q9, _lib.F32, R, 0x1000, RS, 0x2000, US, None, None,
                                   None, None), "neither"),
        (lambda: L.lgb_equilibrium(_lib.D2Q9, _lib.F32, R, 0x1000, RS, 0x2000, US, None, 0x4000,
                                   None, None), "go together"),
        (lambda: L.lgb_init_fneq(_lib.D2Q9, _lib.F32, R, 0x1000, 0x2000, 0.0, 0x3000, None),
         "tau must be positive"),
        (lambda: L.lgb_init_fneq(_lib.D1Q3, _lib.F32, R, 0x1000, 0x2000, 0.6, 0x3000, None),
         "2-D or 3-D"),
        (lambda: L.lgb_init_fneq(_lib.D2Q9, _lib.F32, R, 0x1000, None, 0.6, 0x3000, None),
         "NULL"),
        (lambda: L.lgb_enstrophy(4, _lib.F32, R, 0x1000, 0x2000, 0x3000, None), "dimensions"),
        (lambda: L.lgb_enstrophy(2, _lib.F16_SHIFTED, R, 0x1000, 0x2000, 0x3000, None),
         "precision"),
        (lambda: L.lgb_enstrophy(2, _lib.F32, R, 0x1000, 0x2000, None, None), "NULL"),
    ]
    for call, msg in cases:
        assert call() != 0
        assert msg in L.lgb_last_error().decode(), (msg, L.lgb_last_error())
    bad = _lib.i32x3([0, 6])
    assert L.lgb_enstrophy(2, _lib.F64, ctypes.cast(bad, ctypes.c_void_p), 0x1000, 0x2000,
                           0x3000, None) != 0
    assert "must be positive" in L.lgb_last_error().decode()


@pytest.mark.parametrize("kw,msg", [
    (dict(abi_version=4), "ABI version"),
    (dict(stencil=9), "unknown stencil"),
    (dict(storage=9), "unknown storage"),
    (dict(collision=3), "BGK, TRT or no collision"),
    (dict(n_tiles=0), "empty domain or tile table"),
    (dict(f_out=0x3000), "distinct input and output"),
    (dict(pool_elements=0), "pool_elements must be positive"),
    (dict(threads=48), "a multiple of 32"),
    (dict(blocks=0), "blocks must be positive"),
    (dict(rates=0x4004), "rates must be 16-byte aligned"),
])
def test_batched_step_validation_errors(lgb, kw, msg):
    """lgb_batched_step refuses a bad descriptor before any launch"""
    from lettuce_gb300 import _lib
    from lettuce_gb300._batched import BatchDesc, _bind
    L = _lib.load()
    _bind(L)
    d = BatchDesc()
    d.abi_version = _lib.ABI_VERSION
    d.stencil = _lib.D2Q9
    d.storage = _lib.F32
    d.collision = _lib.BGK
    d.n_domains = 1
    d.n_tiles = 1
    d.threads = 128
    d.blocks = 1
    d.domains = 0x1000
    d.tiles = 0x2000
    d.f_in = 0x3000
    d.f_out = 0x5000
    d.pool_elements = 1024
    for k, v in kw.items():
        setattr(d, k, v)
    rc = L.lgb_batched_step(ctypes.byref(d), None)
    assert rc != 0
    assert msg in L.lgb_last_error().decode()
