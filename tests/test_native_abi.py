"""The C-ABI library builds, loads without a GPU and exports every declared symbol;
the ctypes mirrors of the header's structs have the C layout."""

import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from rkstiff_gb300 import _build, _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rkstiff_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(rk_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    return nat.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert set(names) == set(nat.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", _build.lib_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (rk_\w+)", out))
    for n in names:
        assert n in exported, n
        assert hasattr(lib, n)


def test_abi_version_and_sizes(lib):
    assert lib.rk_abi_version() == nat.ABI_VERSION == 2
    assert lib.rk_num_coeffs(nat.RK_ETD35) == 21
    assert lib.rk_num_coeffs(nat.RK_ETD34) == 10
    assert lib.rk_num_coeffs(nat.RK_IF34) == 2
    assert lib.rk_num_coeffs(nat.RK_IF45DP) == 28
    assert lib.rk_num_coeffs(99) < 0
    # ETD35, FP32, real coefficients, m=513 -> mp=516: 7 complex arrays (the new state shares N2's) and the
    # double-float state's low words of u and of the new state (2 complex arrays), 21 real coefficient arrays
    # and the low word of e^z, the FP32 wavenumbers
    assert lib.rk_slab_bytes(nat.RK_ETD35, nat.RK_FP32, 0, 513) == 9 * 8 * 516 + 22 * 4 * 516 + 4 * 516
    # two coefficient blocks of 22 arrays, then their tags (RK_COEF_BLOCKS_MAX = 4 doubles + 4)
    assert lib.rk_slab_bytes_blocks(nat.RK_ETD35, nat.RK_FP32, 0, 513, 2) == \
        9 * 8 * 516 + 2 * 22 * 4 * 516 + 4 * 516 + 8 * (4 + 4)
    assert lib.rk_slab_bytes(nat.RK_IF34, nat.RK_FP64, 1, 100) == 7 * 16 * 100 + 2 * 16 * 100
    # ETD35 FP32 with complex coefficients: the low word of e^z is a complex array
    assert lib.rk_slab_bytes(nat.RK_ETD35, nat.RK_FP32, 1, 100) == 9 * 8 * 100 + 22 * 8 * 100 + 4 * 100
    assert lib.rk_slab_bytes(nat.RK_ETD35, nat.RK_FP64, 0, 0) < 0


def test_argument_errors_without_gpu(lib):
    b = nat.RkBatch()
    b.method = 42
    assert lib.rk_evolve(ctypes.byref(b), None) == -1
    assert b"unknown method" in lib.rk_last_error()
    assert lib.rk_evolve(None, None) == -1
    b.method = nat.RK_ETD35
    b.precision = 7
    assert lib.rk_evolve(ctypes.byref(b), None) == -1
    b.precision = nat.RK_FP32
    b.n_inst = 0
    assert lib.rk_evolve(ctypes.byref(b), None) == 0  # nothing to do


def test_struct_layout_matches_c():
    """Compile a C probe against the header and compare sizeof/offsetof with ctypes."""
    fields = [f for f, _ in nat.RkBatch._fields_]
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){",
             'printf("%zu %zu %zu %zu\\n", sizeof(rk_batch), sizeof(rk_inst_state), sizeof(rk_controller),'
             ' sizeof(rk_etd_config));']
    for f in fields:
        lines.append(f'printf("%zu\\n", offsetof(rk_batch, {f}));')
    for f in nat.STATE_DTYPE.names:
        lines.append(f'printf("%zu\\n", offsetof(rk_inst_state, {f}));')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(c, "w").write("\n".join(lines))
        subprocess.run(["gcc", "-O0", c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    vals = [int(v) for v in out]
    assert vals[0] == ctypes.sizeof(nat.RkBatch)
    assert vals[1] == nat.STATE_DTYPE.itemsize
    assert vals[2] == ctypes.sizeof(nat.RkController)
    assert vals[3] == ctypes.sizeof(nat.RkEtdConfig)
    offs = vals[4:4 + len(fields)]
    for f, o in zip(fields, offs):
        assert getattr(nat.RkBatch, f).offset == o, f
    soffs = vals[4 + len(fields):]
    for f, o in zip(nat.STATE_DTYPE.names, soffs):
        assert nat.STATE_DTYPE.fields[f][1] == o, f


def test_dense_struct_layout_matches_c():
    """rk_dense_batch / rk_dense_state offsets from the header against the ctypes / NumPy views."""
    fields = [f for f, _ in nat.RkDenseBatch._fields_]
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){",
             'printf("%zu %zu\\n", sizeof(rk_dense_batch), sizeof(rk_dense_state));']
    for f in fields:
        lines.append(f'printf("%zu\\n", offsetof(rk_dense_batch, {f}));')
    for f in nat.DENSE_STATE_DTYPE.names:
        lines.append(f'printf("%zu\\n", offsetof(rk_dense_state, {f}));')
    lines.append('printf("%d %d %d\\n", RK_DENSE_NMAX, RK_DENSE_TILE, RK_NL_ALLEN_CAHN);')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(c, "w").write("\n".join(lines))
        subprocess.run(["gcc", "-O0", c, "-o", exe], check=True)
        vals = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(nat.RkDenseBatch)
    assert vals[1] == nat.DENSE_STATE_DTYPE.itemsize == 128
    offs = vals[2:2 + len(fields)]
    for f, o in zip(fields, offs):
        assert getattr(nat.RkDenseBatch, f).offset == o, f
    soffs = vals[2 + len(fields):2 + len(fields) + len(nat.DENSE_STATE_DTYPE.names)]
    for f, o in zip(nat.DENSE_STATE_DTYPE.names, soffs):
        assert nat.DENSE_STATE_DTYPE.fields[f][1] == o, f
    assert vals[-3:] == [nat.RK_DENSE_NMAX, nat.RK_DENSE_TILE, nat.RK_NL_ALLEN_CAHN]


def test_dense_eig_struct_layout_matches_c():
    """rk_dense_eig_batch offsets from the header against the ctypes view."""
    fields = [f for f, _ in nat.RkDenseEigBatch._fields_]
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){",
             'printf("%zu\\n", sizeof(rk_dense_eig_batch));']
    for f in fields:
        lines.append(f'printf("%zu\\n", offsetof(rk_dense_eig_batch, {f}));')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(c, "w").write("\n".join(lines))
        subprocess.run(["gcc", "-O0", c, "-o", exe], check=True)
        vals = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(nat.RkDenseEigBatch)
    for f, o in zip(fields, vals[1:]):
        assert getattr(nat.RkDenseEigBatch, f).offset == o, f


def _fake_batch(n_inst, n_max):
    """A batch whose device pointers are placeholders: only calls that the host-side checks
    reject may be made with it (nothing dereferences them before those checks)."""
    b = nat.RkBatch()
    b.method = nat.RK_ETD35
    b.precision = nat.RK_FP64
    b.nl_kind = nat.RK_NL_UUX
    b.n_inst = n_inst
    b.n_max = n_max
    for f in ("n", "mode_off", "lin_op", "kx", "u", "state", "twiddle"):
        setattr(b, f, 0x1000)
    b.etd = nat.RkEtdConfig(modecutoff=0.01, contour_radius=1.0, contour_points=32, contour_at_zero=0)
    return b


def test_noalloc_size_check_cannot_overflow(lib):
    """rk_evolve_noalloc bounds the instance count before it multiplies by the slab stride:
    counts whose products wrap int64 are refused, as are counts just past the scratch size.
    Run only where no GPU is present, so that the placeholder pointers can never reach a
    kernel."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("placeholder-pointer checks run on hosts without a GPU")
    stride = (lib.rk_slab_bytes(nat.RK_ETD35, nat.RK_FP64, 0, 2049) + 255) // 256 * 256
    fits = (8 * 2**20 - 511) // (stride + 8)
    for n_inst in (2**63 - 1, 2**63 // stride + 1, (2**64 // stride) // 2, fits + 1, 10**6):
        rc = lib.rk_evolve_noalloc(ctypes.byref(_fake_batch(n_inst, 4096)), None)
        assert rc == nat.RK_E_SIZE, n_inst
        assert b"scratch" in lib.rk_last_error()
    # argument errors are found before the size check, as in rk_evolve
    b = _fake_batch(2, 4096)
    b.kx = None
    assert lib.rk_evolve_noalloc(ctypes.byref(b), None) == nat.RK_E_ARG
    b = _fake_batch(2, 3000)
    assert lib.rk_evolve_noalloc(ctypes.byref(b), None) == nat.RK_E_SIZE
    assert b"power of two" in lib.rk_last_error()


def test_evolve_refuses_the_matrix_contour_flag(lib):
    """contour_at_zero is the matrix-operator form of rk_coeffs; rk_evolve refuses it before
    touching any pointer (so placeholders suffice, and no GPU is needed)."""
    b = _fake_batch(2, 256)
    b.slab = b.slab_off = b.queue = 0x1000
    b.etd = nat.RkEtdConfig(modecutoff=0.01, contour_radius=1.0, contour_points=32, contour_at_zero=1)
    assert lib.rk_evolve(ctypes.byref(b), None) == nat.RK_E_UNSUPPORTED
    assert b"contour_at_zero" in lib.rk_last_error()
