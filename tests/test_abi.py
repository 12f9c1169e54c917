"""The C ABI library: builds, loads, exports what include/gbhf.h declares, and
its ctypes mirror matches the C struct layouts.  No GPU compute here."""
import ctypes as C
import re
import shutil
import subprocess
import textwrap

import pytest

from gbhf import _lib, build


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    syms = _lib.declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_every_exported_entry_point_is_declared(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("nm unavailable")
    exported = set(re.findall(r"\bT (gbhf_[a-z0-9_]+)\b", out.stdout))
    assert exported <= set(_lib.declared_symbols())


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc missing")
def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(textwrap.dedent("""
        #include <stdio.h>
        #include <stddef.h>
        #include "gbhf.h"
        int main(void) {
          printf("%zu %zu %zu %zu %zu\\n", sizeof(gbhf_scf_opts), offsetof(gbhf_scf_opts, conv_error),
                 offsetof(gbhf_scf_opts, charge), sizeof(gbhf_result), offsetof(gbhf_result, fock_builds));
          return 0;
        }"""))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", str(_lib.HEADER.parent), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    want = [C.sizeof(_lib.SCFOpts), _lib.SCFOpts.conv_error.offset, _lib.SCFOpts.charge.offset,
            C.sizeof(_lib.SCFResultC), _lib.SCFResultC.fock_builds.offset]
    assert got == want


def test_option_presets(lib):
    r = _lib.reference_opts()
    assert (r.mode, r.diis_size, r.max_iter, r.conv_error, r.diis_start, r.guess) == (0, 5, 30, 1e-7, 0.1, 0)
    assert r.ref_stop_rule == 1
    b = _lib.baseline_opts()
    assert (b.mode, b.diis_size, b.conv_energy, b.conv_density, b.schwarz_cutoff, b.mixed_cutoff) == \
        (1, 6, 1e-10, 1e-8, 1e-12, 1e-4)


def test_calls_without_gpu_fail_cleanly(lib):
    n = C.c_int(0)
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    assert lib.gbhf_create(C.byref(h), 0) == 6          # GBHF_ERR_NO_DEVICE
    assert lib.gbhf_create(None, 0) == 1                # GBHF_ERR_BAD_INPUT
    assert lib.gbhf_set_basis(None, 0, None, None, 0, None, None, None, None, None) == 1
    assert lib.gbhf_eri_canonical_length(7) == 406
    assert n.value == 0
    with pytest.raises(_lib.GBHFError):
        _lib.Context(0)


HS = _lib.HEADER.parents[1] / "haskell-abinitio_gb300" / "haskell" / "Science" / "QuantumChemistry" / "GPU.hs"


def _c_prototypes():
    text = re.sub(r"/\*.*?\*/", " ", _lib.HEADER.read_text(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(gbhf_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        args = [a for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
        out[m.group(1)] = len(args)
    return out


def test_haskell_binding_matches_the_header():
    """The Haskell module's foreign imports name declared entry points with the
    C argument counts, and its struct offsets are the C layout's."""
    src = HS.read_text()
    protos = _c_prototypes()
    imports = re.findall(r'foreign import ccall (?:safe|unsafe) "(gbhf_[a-z0-9_]+)"\s*\n\s*(\w+)\s*::([^\n]*(?:\n\s+->[^\n]*)*)',
                         src)
    assert len(imports) >= 14
    for cname, hname, ty in imports:
        assert cname in protos, cname
        arrows = ty.count("->")
        assert arrows == max(protos[cname], 1) if protos[cname] else arrows in (0, 1), (cname, arrows, protos[cname])

    def const(name):
        return int(re.search(rf"^{name} = (\d+)$", src, flags=re.M).group(1))

    def lst(name):
        return [int(v) for v in re.search(rf"^{name} = \[([^\]]*)\]", src, flags=re.M).group(1).split(",")]

    o, r = _lib.SCFOpts, _lib.SCFResultC
    names = [f for f, _ in o._fields_]
    assert lst("scfOptsIntOffsets") == [getattr(o, f).offset for f in names[:9]]
    assert lst("scfOptsDoubleOffsets") == [getattr(o, f).offset for f in names[9:17]]
    assert const("scfOptsAutotuneOffset") == o.autotune.offset
    assert const("scfOptsSize") == C.sizeof(o)
    assert const("scfResultSize") == C.sizeof(r)
    for hs_name, field in (("resEnergy", "energy"), ("resIterations", "iterations"), ("resConverged", "converged"),
                           ("resNOccupied", "n_occupied"), ("resFock", "fock_flat"), ("resCoeff", "coeff"),
                           ("resDensity", "density_flat"), ("resOrbE", "orb_energies")):
        assert const(hs_name) == getattr(r, field).offset, hs_name
