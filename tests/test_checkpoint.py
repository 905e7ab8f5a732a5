"""Checkpoint/restart of the design loop: the file format and its checks on
the host, and on the GPU a run restarted from a checkpoint that continues
exactly as the uninterrupted run."""
import struct

import numpy as np
import pytest

import topopt_gb300 as tp


def _fnv1a(data):
    h = 0xCBF29CE484222325
    for b in data:
        h = ((h ^ b) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def _write(path, dims, nrhs, loop, payload):
    nelx, nely, nelz = dims
    ne = nelx * nely * nelz
    nd = 3 * (nelx + 1) * (nely + 1) * (nelz + 1)
    body = np.asarray(payload, np.float64).tobytes()
    hdr = struct.pack("<8s9i2d2qQ", b"TPCKPT1\0", 1, nelx, nely, nelz, 2, nrhs, 1, loop, 0, 0.2, 1.5, ne, nd,
                      _fnv1a(body))
    path.write_bytes(hdr + body)
    return ne, nd


def test_checkpoint_file_checks(tmp_path):
    dims, nrhs = (2, 2, 2), 2
    ne, nd = 8, 3 * 27
    p = tmp_path / "c.bin"
    _write(p, dims, nrhs, 7, np.arange(2 * ne + 2 * nrhs * nd, dtype=np.float64))
    assert tp.checkpoint_info(p) == (2, 2, 2, 2, 2, 1, 7)
    raw = bytearray(p.read_bytes())
    for bad in (raw[:-8], raw + b"\0", raw[:100] + bytes([raw[100] ^ 1]) + raw[101:], b"XPCKPT1\0" + raw[8:]):
        q = tmp_path / "bad.bin"
        q.write_bytes(bytes(bad))
        with pytest.raises(tp.TopOptError):
            tp.checkpoint_info(q)
    with pytest.raises(tp.TopOptError):
        tp.checkpoint_info(tmp_path / "missing.bin")


@pytest.mark.gpu
@pytest.mark.parametrize("nrhs", [1, 2])
def test_restart_continues_the_run(cuda, tmp_path, nrhs):
    shape, nl = (32, 16, 16), 3
    path = tmp_path / "state.bin"

    def make():
        g = tp.TopOpt(*shape, nl, nrhs=nrhs)
        if nrhs > 1:
            g.upload("F", tp.multiload(*shape, nrhs, 4, seed=9).ravel())
        g.init_design()
        return g

    g = make()
    for _ in range(3):
        g.design_iteration()
    g.checkpoint_save(path, 3)
    assert tp.checkpoint_info(path) == shape + (nl, nrhs, tp.TP_FP64, 3)
    ref = [g.design_iteration() for _ in range(2)]
    g.close()
    h = make()  # fresh state (design 0.2, U = 0), then the checkpoint
    assert h.checkpoint_load(path) == 3
    got = [h.design_iteration() for _ in range(2)]
    for a, b in zip(ref, got):
        assert a.c == b.c and a.cgiters == b.cgiters and a.change == b.change
    # a checkpoint of another grid is refused
    w = tp.TopOpt(16, 16, 16, nl, nrhs=nrhs)
    with pytest.raises(tp.TopOptError):
        w.checkpoint_load(path)
    w.close()
    h.close()
