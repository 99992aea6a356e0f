"""The C-ABI library: builds, loads, exports every declared entry point, and its
host-only parts (sampler, validation) behave as the reference.  No GPU needed."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import distembed_gb300 as de

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    from distembed_gb300 import build
    build.build()
    return de.lib()


def _declared():
    names = set()
    for path in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if path.endswith(".h"):
            src = open(os.path.join(ROOT, "include", path)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(de_[a-z0-9_]+)\s*\(", src))
    return names


def test_exports_every_declared_symbol(L):
    declared = _declared()
    assert declared, "no declarations found"
    out = subprocess.run(["nm", "-D", "--defined-only", de.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (de_[a-z0-9_]+)", out))
    assert declared <= exported, declared - exported
    assert set(de.EXPORTS) == declared


def test_version(L):
    assert b"sm_103a" in L.de_version()


def test_default_options(L):
    o = de.Options()
    L.de_default_options(ctypes.byref(o))
    assert (o.precision, o.ref_quirks, o.compute_loss, o.device, o.max_bound) == (0, 1, 1, 0, 5.0)


def test_sampler_matches_reference_golden(L, golden_dir):
    g = np.load(os.path.join(golden_dir, "negatives.npz"))
    assert np.array_equal(de.negatives(60000, 1234, 10), g["u60000_s1234_k10"].astype(np.int64))
    want = g["u4194304_k1024"].astype(np.int64)
    got = np.stack([de.negatives(1 << 22, s, 1024) for s in range(want.shape[0])])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("bad", ["rowptr_start", "rowptr_end", "decreasing", "col_range", "dim"])
def test_create_rejects_bad_input_before_touching_the_gpu(L, bad):
    rowptr = np.array([0, 2, 3, 4], dtype=np.int64)
    col = np.array([1, 2, 0, 1], dtype=np.int64)
    dim = 32
    if bad == "rowptr_start":
        rowptr[0] = 1
    elif bad == "rowptr_end":
        rowptr[-1] = 3
    elif bad == "decreasing":
        rowptr[1:3] = [3, 2]
    elif bad == "col_range":
        col[2] = 3
    else:
        dim = 48
    with pytest.raises(de.DEError) as ei:
        de.Handle(rowptr, col, dim)
    assert ei.value.code == de.DE_ERR_INVALID


@pytest.mark.parametrize("bad", ["rowptr_start", "decreasing", "col_range", "dim", "empty_graph"])
def test_batch_create_rejects_bad_input_before_touching_the_gpu(L, bad):
    rowptr = np.array([0, 2, 3, 4], dtype=np.int64)
    col = np.array([1, 2, 0, 1], dtype=np.int64)
    good = (np.array([0, 1, 2], dtype=np.int64), np.array([1, 0], dtype=np.int64))
    dim = 64
    if bad == "rowptr_start":
        rowptr[0] = 1
    elif bad == "decreasing":
        rowptr[1:3] = [3, 2]
    elif bad == "col_range":
        col[2] = 3
    elif bad == "dim":
        dim = 256
    else:
        rowptr = np.array([0], dtype=np.int64)
    with pytest.raises(de.DEError) as ei:
        de.Batch([good, (rowptr, col)], dim)
    assert ei.value.code == de.DE_ERR_INVALID
