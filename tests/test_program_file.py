"""Program files (tqec_program_save / tqec_program_load).

CPU tests build files in the documented layout here and check that the
loader rejects what is not a program file (missing: TQEC_ERR_IO; foreign,
truncated, corrupted, malformed network: TQEC_ERR_INVALID), and that a well-formed
file gets through parsing and the network checks to the point where a
device is needed.  The GPU test saves an autotuned program, loads it, and
requires the same launch shapes and bit-identical decodes.
"""
import struct

import numpy as np
import pytest

from conftest import gpu_available

MAGIC = b"TQECPROG"


def _fnv1a(data, h=0xcbf29ce484222325):
    for b in data:
        h ^= b
        h = (h * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h


def _vec(a, fmt):
    a = np.ascontiguousarray(a, dtype=fmt)
    return struct.pack("<Q", a.size) + a.tobytes()


def _shape(G=1, threads=128, smem_arena=1, smem_tables=0, split=0, tensor=0, smem=4096, grid_cap=152):
    return struct.pack("<iiBBBBQi", G, threads, smem_arena, smem_tables, split, tensor, smem, grid_cap)


def program_file(graph, steps, precision=1, flags=0, device=0, tamper=None):
    """Bytes of a program file for `graph` compiled along `steps` (launch
    shapes and fingerprint are placeholders: a loader on a GPU would reject
    the fingerprint, which the CPU tests never reach)."""
    ix_off, labels, d_off, data, iy, synd = graph.flat()
    fields = {
        "head": MAGIC + struct.pack("<II", 1, 0x01020304),
        "opts": struct.pack("<iIiiidi", precision, flags, device, 0, 0, -1.0, 0),
        "n": struct.pack("<i", graph.n_tensors),
        "ix_off": _vec(ix_off, "<i4"), "labels": _vec(labels, "<i4"), "d_off": _vec(d_off, "<i8"),
        "data": _vec(data, "<f8"), "iy": _vec(iy, "<i4"), "synd": _vec(synd, "<i4"),
        "steps": _vec(np.asarray(steps).reshape(-1), "<i4"),
        "tail": struct.pack("<QiQ", 0, 152, 232448)
        + b"".join(_shape() + struct.pack("<i", 0) for _ in range(3)) + _shape(),
    }
    if tamper:
        tamper(fields)
    body = b"".join(fields.values())
    return body + struct.pack("<Q", _fnv1a(body))


def _load(pkg, path):
    import ctypes as C

    h = C.c_void_p()
    rc = pkg.native.lib().tqec_program_load(str(path).encode(), -1, C.byref(h))
    return rc, pkg.native.last_error()


def _graph(pkg):
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.depolarizing(0.05, t.nq)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    return g, pkg.optimize_code(g, pkg.GreedyMethod())


def test_loader_rejects_what_is_not_a_program_file(pkg, tmp_path):
    g, steps = _graph(pkg)
    good = program_file(g, steps)
    cases = {
        "missing": None,
        "foreign": b"\x7fELF" + bytes(200),
        "truncated": good[:-20],
        "corrupted": good[:100] + bytes([good[100] ^ 1]) + good[101:],
    }
    for name, data in cases.items():
        path = tmp_path / name
        if data is not None:
            path.write_bytes(data)
        rc, msg = _load(pkg, path)
        assert rc == (-6 if data is None else -1), (name, rc, msg)  # TQEC_ERR_IO / TQEC_ERR_INVALID
    rc, msg = _load(pkg, tmp_path / "corrupted")
    assert "checksum" in msg


@pytest.mark.parametrize("what", ["offsets", "steps", "version", "extra"])
def test_loader_rejects_malformed_contents(pkg, tmp_path, what):
    g, steps = _graph(pkg)

    def tamper(f):
        if what == "offsets":  # label offsets that run past the label array
            ix = np.frombuffer(f["ix_off"][8:], dtype="<i4").copy()
            ix[-1] += 5
            f["ix_off"] = _vec(ix, "<i4")
        elif what == "steps":  # one step short of a tree
            f["steps"] = _vec(np.asarray(steps).reshape(-1)[:-2], "<i4")
        elif what == "version":
            f["head"] = MAGIC + struct.pack("<II", 2, 0x01020304)
        else:  # bytes after the last field
            f["tail"] += b"\0" * 4

    path = tmp_path / "bad"
    path.write_bytes(program_file(g, steps, tamper=tamper))
    rc, msg = _load(pkg, path)
    assert rc == -1, (rc, msg)


@pytest.mark.skipif(gpu_available(), reason="checks the CPU-only path up to the device")
def test_well_formed_file_reaches_the_device(pkg, tmp_path):
    g, steps = _graph(pkg)
    path = tmp_path / "ok"
    path.write_bytes(program_file(g, steps))
    rc, msg = _load(pkg, path)
    # parsing and the network checks passed; creating the program needs a GPU
    assert rc == -2, (rc, msg)  # TQEC_ERR_CUDA
    assert "program file" not in msg and "malformed" not in msg


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")
def test_save_load_roundtrip_on_gpu(pkg, tmp_path):
    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    em = pkg.depolarizing(0.08, t.nq)
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    prog = ct.program
    prog.autotune(4096)
    path = tmp_path / "surface5.tqec"
    prog.save(str(path))
    loaded = pkg.native.Program.load(str(path))
    assert loaded.info == prog.info
    assert (loaded.precision, loaded.flags) == (prog.precision, prog.flags)
    rng = np.random.default_rng(21)
    ep = pkg.random_error_pattern(em, rng, nsamples=3000)
    s = pkg.syndrome_extraction(ep, t)
    packed = pkg.pack_syndromes(np.concatenate([s.sx, s.sz], axis=1))
    nc = prog.n_classes
    lp_a, lp_b = np.empty((3000, nc)), np.empty((3000, nc))
    cls_a = prog.decode_packed(packed, logp=lp_a)
    cls_b = loaded.decode_packed(packed, logp=lp_b)
    np.testing.assert_array_equal(cls_a, cls_b)
    np.testing.assert_array_equal(lp_a, lp_b)
    # a loaded program saves the same file again
    again = tmp_path / "again.tqec"
    loaded.save(str(again))
    assert again.read_bytes() == path.read_bytes()
    loaded.close()
    ct.close()
    data = path.read_bytes()
    bad = tmp_path / "bad.tqec"
    bad.write_bytes(data[:200] + bytes([data[200] ^ 1]) + data[201:])
    with pytest.raises(pkg.native.TqecError):
        pkg.native.Program.load(str(bad))
