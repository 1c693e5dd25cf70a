"""On-disk formats (host only, no GPU): result.bin / initial.bin as the reference writes and reads
them, the ghost-slab layout of the reference's multi-GPU files, and the CRC-checked state
snapshot used to resume runs."""
import ctypes as C
import zlib

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def test_crc32_matches_the_standard_check_value_and_zlib(native):
    assert native.adv_crc32(b"123456789", 9) == 0xCBF43926
    data = np.random.default_rng(0).integers(0, 256, 10007, dtype=np.uint8).tobytes()
    assert native.adv_crc32(data, len(data)) == zlib.crc32(data)


def test_result_bin_round_trip_and_size_check(native, tmp_path):
    u = np.random.default_rng(1).standard_normal(7 * 5 * 3)
    path = str(tmp_path / "result.bin").encode()
    assert native.adv_write_result_bin(path, N.ADV_F64, u.ctypes.data, u.size) == N.ADV_OK
    # the reference's reader: fread(fID, [1, nx*ny*nz], 'float')
    np.testing.assert_array_equal(np.fromfile(path.decode(), dtype=np.float32), u.astype(np.float32))
    back = np.empty_like(u)
    assert native.adv_read_result_bin(path, u.size, _dp(back)) == N.ADV_OK
    np.testing.assert_array_equal(back, u.astype(np.float32).astype(np.float64))
    assert native.adv_read_result_bin(path, u.size + 1, _dp(np.empty(u.size + 1))) == N.ADV_ERR_INVALID_ARG
    assert b"expected" in native.adv_last_error_string()


@pytest.mark.parametrize("periodic", [0, 1])
def test_ghost_slabs_pad_and_strip(native, periodic):
    nx, ny, nz, R = 4, 3, 8, 3
    interior = np.arange(nx * ny * nz, dtype=np.float64)
    ghosted = np.full(nx * ny * (nz + 2 * R), -1.0)
    assert native.adv_pad_ghost_slabs(nx, ny, nz, R, periodic, _dp(interior), _dp(ghosted)) == N.ADV_OK
    g = ghosted.reshape(nz + 2 * R, ny, nx)
    i = interior.reshape(nz, ny, nx)
    np.testing.assert_array_equal(g[R:R + nz], i)
    if periodic:
        np.testing.assert_array_equal(g[:R], i[nz - R:])
        np.testing.assert_array_equal(g[R + nz:], i[:R])
    else:
        assert not g[:R].any() and not g[R + nz:].any()
    back = np.empty_like(interior)
    assert native.adv_strip_ghost_slabs(nx, ny, nz, R, _dp(ghosted), _dp(back)) == N.ADV_OK
    np.testing.assert_array_equal(back, interior)


@pytest.mark.parametrize("dtype,code", [(np.float32, N.ADV_F32), (np.float64, N.ADV_F64)])
def test_checkpoint_round_trip(native, tmp_path, dtype, code):
    nx, ny, nz = 9, 7, 5
    u = np.random.default_rng(2).standard_normal(nx * ny * nz).astype(dtype)
    path = str(tmp_path / "state.bin").encode()
    assert native.adv_checkpoint_save(path, code, nx, ny, nz, 1234, 0.375, u.ctypes.data) == N.ADV_OK
    h = N.CheckpointHeader()
    assert native.adv_checkpoint_load(path, C.byref(h), None, 0) == N.ADV_OK  # header only
    assert (h.version, h.dtype, h.nx, h.ny, h.nz, h.step, h.t) == (1, code, nx, ny, nz, 1234, 0.375)
    assert h.payload_bytes == u.nbytes and h.payload_crc32 == zlib.crc32(u.tobytes())
    back = np.empty_like(u)
    assert native.adv_checkpoint_load(path, C.byref(h), back.ctypes.data, back.nbytes) == N.ADV_OK
    np.testing.assert_array_equal(back, u)
    assert native.adv_checkpoint_load(path, C.byref(h), back.ctypes.data, back.nbytes - 1) == N.ADV_ERR_INVALID_ARG


def test_checkpoint_rejects_damaged_files(native, tmp_path):
    nx, ny, nz = 6, 5, 4
    u = np.random.default_rng(3).standard_normal(nx * ny * nz)
    good = tmp_path / "state.bin"
    assert native.adv_checkpoint_save(str(good).encode(), N.ADV_F64, nx, ny, nz, 7, 1.5, u.ctypes.data) == N.ADV_OK
    raw = good.read_bytes()
    h = N.CheckpointHeader()
    back = np.empty_like(u)

    def load(data, name):
        p = tmp_path / name
        p.write_bytes(data)
        st = native.adv_checkpoint_load(str(p).encode(), C.byref(h), back.ctypes.data, back.nbytes)
        return st, native.adv_last_error_string().decode()

    flipped = bytearray(raw)
    flipped[128 + 17] ^= 0x01  # one bit of the payload
    assert load(bytes(flipped), "payload.bin") == (N.ADV_ERR_INVALID_ARG, "checkpoint_load: payload CRC mismatch")
    flipped = bytearray(raw)
    flipped[33] ^= 0x10  # the step count
    assert load(bytes(flipped), "header.bin") == (N.ADV_ERR_INVALID_ARG, "checkpoint_load: header CRC mismatch")
    assert load(raw[:-8], "short.bin") == (N.ADV_ERR_INVALID_ARG, "checkpoint_load: truncated payload")
    assert load(raw + b"\x00", "appended.bin") == (N.ADV_ERR_INVALID_ARG, "checkpoint_load: data after the payload")
    assert load(raw + raw, "joined.bin") == (N.ADV_ERR_INVALID_ARG, "checkpoint_load: data after the payload")
    assert load(raw, "intact.bin")[0] == N.ADV_OK
    np.testing.assert_array_equal(back, u)
    assert load(raw[:100], "stub.bin") == (N.ADV_ERR_INVALID_ARG, "checkpoint_load: truncated header")
    assert load(b"NOTSTATE" + raw[8:], "magic.bin") == (N.ADV_ERR_INVALID_ARG,
                                                        "checkpoint_load: not a state snapshot")
    assert not (tmp_path / "state.bin.tmp").exists()  # saved through a temporary name and a rename
