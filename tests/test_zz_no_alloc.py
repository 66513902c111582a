"""ffg_pauli_rotations_noalloc: the allocation-free entry point for callers that
cannot allocate device memory when they call it (processes whose device
memory a framework's caching allocator already holds, loops that must not
trigger cudaFree's device-wide synchronisation).  It keeps its term store in a
fixed device array inside libffg; these tests check that its output equals the
context-based ffg_pauli_propagate entry point and the CPU oracle on two calls
in a row, that it leaves the device's free memory unchanged, and that sizes
beyond the fixed limit, a too-small output, and duplicate keys are reported.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

import fastfermion_gb300 as ff
from fastfermion_gb300 import _native
from golden_io import assert_same_terms
from oracle import oracle as O

pytestmark = pytest.mark.gpu

LIMIT_IN = 32768


def _circuit(seed, nq_sets):
    rng = np.random.default_rng(seed)
    circ = []
    for _ in range(36):
        w = int(rng.integers(1, 4))
        qs = sorted(int(q) for q in rng.choice(nq_sets, w, replace=False))
        circ.append(ff.ROT("".join("XYZ"[rng.integers(3)] for _ in qs), qs, float(rng.uniform(-2, 2))))
    obs = ff.PauliPolynomial(ff.PauliString([(int(nq_sets[0]), "Z")]), 0.7 + 0.2j)
    obs = obs + ff.PauliPolynomial(ff.PauliString([(int(nq_sets[-1]), "X"), (int(nq_sets[1]), "Y")]), -1.3)
    return circ, obs


def _noalloc(torch, keys, re, im, table, maxdegree, out_cap=65536, free_delta=None):
    L = _native.lib()
    n = re.size
    dk = torch.from_numpy(keys.astype(np.int64)).cuda().contiguous()
    dre = torch.from_numpy(re).cuda()
    dim = torch.from_numpy(im).cuda() if im is not None else None
    ok = torch.zeros((4, out_cap), dtype=torch.int64, device="cuda")
    ore = torch.zeros(out_cap, dtype=torch.float64, device="cuda")
    oim = torch.zeros(out_cap, dtype=torch.float64, device="cuda")
    n_out = ctypes.c_size_t(0)
    err = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = L.ffg_pauli_rotations_noalloc(
        ctypes.c_void_p(stream), ctypes.c_void_p(dk.data_ptr()), ctypes.c_void_p(dre.data_ptr()),
        ctypes.c_void_p(dim.data_ptr() if dim is not None else None), n, table.ctypes.data_as(ctypes.c_void_p), table.size,
        int(maxdegree), ctypes.c_void_p(ok.data_ptr()), ctypes.c_void_p(ore.data_ptr()),
        ctypes.c_void_p(oim.data_ptr()), out_cap, ctypes.byref(n_out), err, 256)
    if free_delta is not None:
        free_delta.append(free0 - torch.cuda.mem_get_info()[0])
    m = min(n_out.value, out_cap)
    keys_out = ok[:, :m].cpu().numpy().astype(np.uint64)
    return rc, err.value.decode(), (keys_out, ore[:m].cpu().numpy(), oim[:m].cpu().numpy())


def _reference_entry(keys, re, im, table, maxdegree):
    ctx = _native.context(0)
    r = ctx.pauli_propagate(keys, re, im, table, dict(maxdegree=maxdegree, topk=0, mincoeff=0.0,
                                                      max_xweight=-1, xtrunc_period=1, batched=0,
                                                      deterministic=0))
    return r.copy()


def test_noalloc_matches_propagate_two_calls():
    torch = pytest.importorskip("torch")
    cases = [_circuit(11, [0, 1, 2, 3, 4, 5, 6]), _circuit(12, [0, 7, 63, 64, 65, 100, 127])]
    for circ, obs in cases:  # two calls in a row, different inputs
        table = ff.encode_pauli_circuit(circ)
        keys, re, im = obs.arrays()
        rc, msg, got = _noalloc(torch, keys, re, im, table, maxdegree=5)
        assert rc == 0, msg
        want = _reference_entry(keys, re, im, table, 5)
        assert got[0].shape[1] == want[0].shape[1]
        assert_same_terms(got, want)  # bit-identical coefficients (==)
        o = O.pauli_propagate(table, keys, re, im, maxdegree=5, batched=False)
        assert_same_terms(got, (o.keys, o.re, o.im))


def test_noalloc_allocates_nothing_and_takes_null_imaginary_parts():
    torch = pytest.importorskip("torch")
    circ, obs = _circuit(13, [0, 2, 5, 9, 64, 70])
    table = ff.encode_pauli_circuit(circ)
    keys, re, _ = obs.arrays()
    re = re.real.copy() if np.iscomplexobj(re) else re
    rc, msg, first = _noalloc(torch, keys, re, None, table, maxdegree=4)
    assert rc == 0, msg
    delta = []
    rc, msg, again = _noalloc(torch, keys, re, None, table, maxdegree=4, free_delta=delta)
    assert rc == 0, msg
    assert delta == [0]  # the device's free memory is unchanged across the call
    assert_same_terms(again, first)
    o = O.pauli_propagate(table, keys, re, np.zeros_like(re), maxdegree=4, batched=False)
    assert_same_terms(again, (o.keys, o.re, o.im))


def test_noalloc_reports_size_when_output_is_too_small():
    torch = pytest.importorskip("torch")
    circ, obs = _circuit(14, [1, 3, 4, 8])
    table = ff.encode_pauli_circuit(circ)
    keys, re, im = obs.arrays()
    rc, msg, full = _noalloc(torch, keys, re, im, table, maxdegree=6)
    assert rc == 0, msg
    need = full[0].shape[1]
    assert need > 2
    L = _native.lib()
    n_out = ctypes.c_size_t(0)
    err = ctypes.create_string_buffer(256)
    dk = torch.from_numpy(keys.astype(np.int64)).cuda().contiguous()
    dre, dim = torch.from_numpy(re).cuda(), torch.from_numpy(im).cuda()
    ok = torch.zeros((4, 2), dtype=torch.int64, device="cuda")
    ore = torch.zeros(2, dtype=torch.float64, device="cuda")
    oim = torch.zeros(2, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = L.ffg_pauli_rotations_noalloc(
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), ctypes.c_void_p(dk.data_ptr()),
        ctypes.c_void_p(dre.data_ptr()), ctypes.c_void_p(dim.data_ptr()), re.size,
        table.ctypes.data_as(ctypes.c_void_p), table.size, 6, ctypes.c_void_p(ok.data_ptr()),
        ctypes.c_void_p(ore.data_ptr()), ctypes.c_void_p(oim.data_ptr()), 2, ctypes.byref(n_out), err, 256)
    assert rc == -1 and "out_cap" in err.value.decode()
    assert n_out.value == need


def test_noalloc_rejects_duplicate_keys():
    torch = pytest.importorskip("torch")
    keys = np.zeros((4, 2), dtype=np.uint64)
    keys[2, :] = 5  # the same string twice
    table = ff.encode_pauli_circuit([ff.ROT("X", [0], 0.4)])
    rc, msg, _ = _noalloc(torch, keys, np.ones(2), np.zeros(2), table, 128)
    assert rc == -1 and "duplicate" in msg


def test_noalloc_rejects_oversized_input():
    torch = pytest.importorskip("torch")
    n = LIMIT_IN + 1
    keys = np.zeros((4, n), dtype=np.uint64)
    keys[2] = np.arange(n, dtype=np.uint64) + 1
    rc, msg, _ = _noalloc(torch, keys, np.ones(n), np.zeros(n), np.zeros(0, dtype=_native.PAULI_GATE), 128)
    assert rc == -1 and "exceed the fixed scratch limit" in msg


def test_noalloc_reports_growth_past_limit():
    torch = pytest.importorskip("torch")
    # 17 single-qubit X rotations on a 17-qubit Z string double the term count each
    obs = ff.PauliString("Z" * 17)
    circ = [ff.ROT("X", [q], 0.3) for q in range(17)]
    keys, re, im = ff.PauliPolynomial(obs).arrays()
    rc, msg, _ = _noalloc(torch, keys, re, im, ff.encode_pauli_circuit(circ), 128)
    assert rc == -1 and "outgrew the fixed scratch limit" in msg
    # the message names the caller's gates[] index: the store holds 2^k terms
    # after k rotations (applied last gate first), and a rotation is refused
    # when it could double the store past 2^16 terms: the 17th applied, gates[0]
    assert "at gates[0]" in msg
