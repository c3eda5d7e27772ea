"""The render loop's files (nerf/main/render.py:27-117) on the host: the PNG
encoder against an independent decoder, the file names, and the loop's
outputs with a stand-in renderer (the device calls the loop makes,
NeRF.render_frame and create_depth_map, have their own GPU tests)."""
import importlib
import os
import struct
import zlib

import numpy as np
import pytest
import torch


def decode_png(path):
    """Minimal PNG decoder for 8-bit, non-interlaced RGB/grey files with any
    of the five row filters (PNG specification, ISO/IEC 15948, 9.2)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(kind + body) & 0xFFFFFFFF, kind
        chunks.append((kind, body))
        pos += 12 + n
    assert chunks[0][0] == b"IHDR" and chunks[-1][0] == b"IEND"
    W, H, depth, colour, comp, filt, lace = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, comp, filt, lace) == (8, 0, 0, 0) and colour in (0, 2)
    bpp = 3 if colour == 2 else 1
    raw = zlib.decompress(b"".join(b for k, b in chunks if k == b"IDAT"))
    stride = W * bpp
    out = np.zeros((H, stride), np.int64)
    prev = np.zeros(stride, np.int64)
    for y in range(H):
        ftype = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int64)
        cur = np.zeros(stride, np.int64)
        for x in range(stride):
            a = cur[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if ftype == 0:
                pred = 0
            elif ftype == 1:
                pred = a
            elif ftype == 2:
                pred = b
            elif ftype == 3:
                pred = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            cur[x] = (line[x] + pred) & 0xFF
        out[y], prev = cur, cur
    img = out.astype(np.uint8)
    return img.reshape(H, W, 3) if colour == 2 else img


@pytest.mark.parametrize("shape", [(7, 5, 3), (1, 1, 3), (64, 33), (3, 200, 3)])
def test_write_png_roundtrip(ng, tmp_path, shape):
    rl = importlib.import_module("nerf-tf2_gb300.render_loop")
    img = np.random.default_rng(sum(shape)).integers(0, 256, shape, dtype=np.uint8)
    p = str(tmp_path / "x.png")
    rl.write_png(p, img)
    assert np.array_equal(decode_png(p), img)


def test_write_png_rejects(ng, tmp_path):
    rl = importlib.import_module("nerf-tf2_gb300.render_loop")
    for bad in (np.zeros((4, 4, 3), np.float32), np.zeros((4, 4, 4), np.uint8), np.zeros((0, 4, 3), np.uint8),
                np.zeros(5, np.uint8)):
        with pytest.raises(ValueError):
            rl.write_png(str(tmp_path / "bad.png"), bad)


def test_render_name(ng):
    rl = importlib.import_module("nerf-tf2_gb300.render_loop")
    # render.py:76: zfill = int(log10(num_cameras) + 5)
    assert rl.render_name(0, 1) == "render_00000"
    assert rl.render_name(3, 9) == "render_00003"
    assert rl.render_name(12, 10) == "render_000012"
    assert rl.render_name(7, 120) == "render_0000007"


def test_render_cameras_files(ng, tmp_path, monkeypatch):
    """Directories, names and contents of the loop's files (render.py:27-117)
    with a stand-in renderer and depth-map function on the host."""
    rl = importlib.import_module("nerf-tf2_gb300.render_loop")
    H, W = 6, 9
    calls, frames = [], []

    class FakeNeRF:
        def render_frame(self, H_, W_, intrinsic, c2w, bounds, **kw):
            calls.append((H_, W_, bounds, kw))
            g = torch.Generator().manual_seed(len(calls))
            rgb = torch.rand(H_, W_, 3, generator=g)
            frames.append({"rgb": rgb, "depth": 2.0 + 4.0 * torch.rand(H_, W_, generator=g),
                           "acc": torch.rand(H_, W_, generator=g),
                           "image_u8": (rgb * 255.0).clamp(0.0, 255.0).to(torch.uint8)})
            return frames[-1]

    def fake_depth(pred_depth, H_, W_, scale_factor, map_type, intrinsic=None, C_to_W2=None):
        d = pred_depth.reshape(H_, W_)
        if map_type == "type_1":
            assert intrinsic is None and C_to_W2 is None
            return d / scale_factor
        assert intrinsic is not None and C_to_W2 is not None
        return d * 0.5

    monkeypatch.setattr(rl.ray_utils, "create_depth_map", fake_depth)
    poses = [np.eye(4), np.eye(4) * 2.0, np.eye(4) * 3.0]
    names = rl.render_cameras(FakeNeRF(), poses, np.eye(3), H, W, (2.0, 6.0), str(tmp_path), scale_factor=0.25,
                              seed=11, chunk=64)
    assert names == ["render_00000", "render_00001", "render_00002"]
    assert calls == [(H, W, (2.0, 6.0), {"seed": 11, "chunk": 64})] * 3
    assert sorted(os.listdir(tmp_path)) == sorted(rl.SUBDIRS)
    for name, fr in zip(names, frames):
        assert np.array_equal(decode_png(str(tmp_path / "rgb" / f"{name}.png")), fr["image_u8"].numpy())
        d1 = np.load(tmp_path / "depth_type_1" / f"{name}.npy")
        d2 = np.load(tmp_path / "depth_type_2" / f"{name}.npy")
        acc = np.load(tmp_path / "acc_map" / f"{name}.npy")
        assert d1.shape == d2.shape == acc.shape == (H, W)
        np.testing.assert_array_equal(d1, (fr["depth"] / 0.25).numpy())
        np.testing.assert_array_equal(d2, (fr["depth"] * 0.5).numpy())
        np.testing.assert_array_equal(acc, fr["acc"].numpy())


@pytest.mark.parametrize("n,inc", [(1, 60.0), (7, 45.0), (40, 80.0)])
def test_create_spherical_path(ng, tmp_path, n, inc):
    """pose_utils.py:770-840: the same pose as synthetic.look_at_pose per
    camera; cameras on the sphere, looking at the origin, right-handed
    orthonormal frames (to the 1e-8 of the reference's normalisation),
    azimuths 360/n degrees apart; the manual rotation left-multiplies every
    pose."""
    rl = importlib.import_module("nerf-tf2_gb300.render_loop")
    poses = rl.create_spherical_path(4.0, inc, n)
    assert poses.shape == (n, 4, 4) and poses.dtype == np.float64
    for i in range(n):
        want = ng.synthetic.look_at_pose(np.radians(360.0 * i / n), np.radians(inc), 4.0)
        np.testing.assert_allclose(poses[i], want, rtol=0, atol=1e-14)
        R, t = poses[i, :3, :3], poses[i, :3, 3]
        # unit to within the reference's normalisation epsilon (|v| + 1e-8)
        np.testing.assert_allclose(R.T @ R, np.eye(3), rtol=0, atol=1e-7)
        assert abs(np.linalg.det(R) - 1.0) < 1e-7
        np.testing.assert_allclose(np.linalg.norm(t), 4.0, rtol=1e-15)
        np.testing.assert_allclose(R[:, 2], -t / np.linalg.norm(t), atol=1e-8)
        np.testing.assert_allclose(np.degrees(np.arccos(t[2] / 4.0)), inc, atol=1e-9)
    assert np.array_equal(poses[:, 3], np.tile([0.0, 0.0, 0.0, 1.0], (n, 1)))
    c, s_ = np.cos(0.3), np.sin(0.3)
    rot = np.array([[c, -s_, 0.0], [s_, c, 0.0], [0.0, 0.0, 1.0]])
    np.save(tmp_path / "rot.npy", rot)
    turned = rl.create_spherical_path(4.0, inc, n, manual_rotation=str(tmp_path / "rot.npy"))
    T = np.eye(4)
    T[:3, :3] = rot
    np.testing.assert_array_equal(turned, T @ poses)
    assert rl.default_bounds(4.0) == (2.0, 6.0)
