"""The render loop's files (nerf/main/render.py:27-117) without OpenCV.

Per camera pose the reference renders one frame and writes, under its save
directory, ``rgb/<name>.png`` (the 8-bit image, render.py:95-100),
``depth_type_1/<name>.npy`` and ``depth_type_2/<name>.npy`` (the depth maps,
:102-113) and ``acc_map/<name>.npy`` (:115-117). The PNG encoder here uses
only the standard library (zlib and its CRC-32).
"""
import os
import struct
import zlib

import numpy as np

from . import ray_utils
from .synthetic import _normalize

# render.py:28-31
SUBDIRS = ("rgb", "acc_map", "depth_type_1", "depth_type_2")


def _png_chunk(kind, data):
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def write_png(path, image):
    """An 8-bit PNG of `image`, uint8 [H, W, 3] (RGB) or [H, W] (grey).

    The file is the PNG signature, an IHDR chunk (bit depth 8, colour type 2
    or 0, no interlace), one zlib-compressed IDAT of the rows, each prefixed
    with filter type 0, and IEND (PNG specification, ISO/IEC 15948). The
    reference's cv2.imwrite (render.py:99-100) stores the same pixels with
    its own filters and compression level, so the files differ in bytes but
    not in the image they decode to."""
    a = np.ascontiguousarray(np.asarray(image))
    if a.dtype != np.uint8 or a.ndim not in (2, 3) or (a.ndim == 3 and a.shape[2] != 3):
        raise ValueError(f"expected uint8 [H, W, 3] or [H, W], got {a.dtype} {a.shape}")
    H, W = a.shape[:2]
    if H == 0 or W == 0:
        raise ValueError("empty image")
    colour = 2 if a.ndim == 3 else 0
    rows = a.reshape(H, -1)
    raw = b"".join(b"\x00" + rows[y].tobytes() for y in range(H))
    png = (b"\x89PNG\r\n\x1a\n" + _png_chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, 8, colour, 0, 0, 0)) +
           _png_chunk(b"IDAT", zlib.compress(raw, 6)) + _png_chunk(b"IEND", b""))
    with open(path, "wb") as f:
        f.write(png)


def create_spherical_path(radius, inclination, num_cameras, manual_rotation=None):
    """The render loop's cameras (pose_utils.py:770-840): num_cameras
    camera-to-world poses [N, 4, 4] (float64) on a sphere of `radius` about
    the origin, at `inclination` degrees from +z and azimuths evenly spaced
    over [0, 360) degrees. Each camera's z axis points at the origin, its x
    axis along the azimuthal direction, y = z x x. `manual_rotation`: None,
    or the path of a .npy 3x3 rotation applied to every pose (rotation @
    pose)."""
    az = np.radians(np.linspace(0, 360, num_cameras, endpoint=False, dtype=np.float64))
    inc = np.radians(np.full_like(az, inclination))
    r = np.full_like(az, radius)
    origins = np.stack([r * np.sin(inc) * np.cos(az), r * np.sin(inc) * np.sin(az), r * np.cos(inc)], axis=1)
    z = _normalize(-1 * origins)
    x = _normalize(np.stack([-1 * r * np.sin(inc) * np.sin(az), r * np.sin(inc) * np.cos(az), np.zeros_like(az)],
                            axis=1))
    y = _normalize(np.cross(z, x))
    poses = np.zeros((num_cameras, 4, 4), dtype=np.float64)
    poses[:, :3, 0], poses[:, :3, 1], poses[:, :3, 2], poses[:, :3, 3] = x, y, z, origins
    poses[:, 3, 3] = 1.0
    if manual_rotation is not None:
        transform = np.eye(4, dtype=np.float64)
        transform[:3, :3] = np.load(manual_rotation)
        poses = transform @ poses
    return poses


def default_bounds(radius):
    """render.py:64-71: without configured bounds, near and far are 25 % and
    75 % of the sphere's diameter."""
    diameter = 2 * radius
    return (0.25 * diameter, 0.75 * diameter)


def render_name(i, num_cameras):
    """render.py:76 and :88: ``render_`` + the camera index zero-filled to
    int(log10(num_cameras) + 5) digits."""
    return f"render_{str(i).zfill(int(np.log10(num_cameras) + 5))}"


def render_cameras(nerf, poses, intrinsic, H, W, bounds, save_dir, scale_factor=1.0, **render_kw):
    """The render loop (render.py:79-117): for every camera-to-world pose,
    NeRF.render_frame (rays from the pinhole camera on the device, the
    render in chunks; keyword arguments pass through) and the four files
    under `save_dir`. `scale_factor` is the dataset's adjusted scale factor
    (render.py:63), which divides the type-1 depth. Returns the names."""
    for sub in SUBDIRS:
        os.makedirs(os.path.join(save_dir, sub), exist_ok=True)
    names = []
    for i, c2w in enumerate(poses):
        frame = nerf.render_frame(H, W, intrinsic, c2w, bounds=bounds, **render_kw)
        name = render_name(i, len(poses))
        write_png(os.path.join(save_dir, "rgb", name + ".png"), frame["image_u8"].cpu().numpy())
        depth = frame["depth"].reshape(-1)
        d1 = ray_utils.create_depth_map(depth, H, W, scale_factor, "type_1")
        d2 = ray_utils.create_depth_map(depth, H, W, scale_factor, "type_2", intrinsic=intrinsic, C_to_W2=c2w)
        np.save(os.path.join(save_dir, "depth_type_1", name + ".npy"), d1.cpu().numpy())
        np.save(os.path.join(save_dir, "depth_type_2", name + ".npy"), d2.cpu().numpy())
        np.save(os.path.join(save_dir, "acc_map", name + ".npy"), frame["acc"].reshape(H, W).cpu().numpy())
        names.append(name)
    return names
