"""Point clouds: the host-side container and its file formats.

``CvoPointCloud`` mirrors the fields of the reference's cloud container
(include/UnifiedCvo/utils/CvoPointCloud.hpp:32-221) that the registration path
reads: positions, an F-dimensional feature vector, a C-class label
distribution and the 2-vector geometric type.  It is stored as packed float32
arrays (structure of arrays) instead of the reference's 176-240 byte records.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import CvoCloudC


class CvoPointCloud:
    """Point cloud with optional features (F), label distributions (C) and geometric types."""

    def __init__(self, xyz, features=None, labels=None, geom_type=None):
        xyz = np.ascontiguousarray(np.asarray(xyz, dtype=np.float32).reshape(-1, 3))
        n = xyz.shape[0]
        self.xyz = xyz
        self.features = None if features is None else self._rows(features, n)
        self.labels = None if labels is None else self._rows(labels, n)
        self.geom_type = None if geom_type is None else np.ascontiguousarray(np.asarray(geom_type, np.float32).reshape(n, 2))

    @staticmethod
    def _rows(a, n):
        """(n, k) float32; an empty cloud keeps the column count of a 2-D input."""
        a = np.asarray(a, np.float32)
        k = a.shape[1] if a.ndim == 2 else (a.size // n if n else 0)
        return np.ascontiguousarray(a.reshape(n, k))

    # -- sizes (CvoPointCloud::num_points / feature_dimensions / num_classes)
    def num_points(self) -> int:
        return int(self.xyz.shape[0])

    def feature_dimensions(self) -> int:
        return 0 if self.features is None else int(self.features.shape[1])

    def num_classes(self) -> int:
        return 0 if self.labels is None else int(self.labels.shape[1])

    def __len__(self) -> int:
        return self.num_points()

    def c_struct(self) -> CvoCloudC:
        """C-ABI descriptor; the arrays stay owned by this object."""
        fp = C.POINTER(C.c_float)
        c = CvoCloudC()
        c.n = self.num_points()
        c.F = self.feature_dimensions()
        c.C = self.num_classes()
        c.xyz_stride = 3
        c.xyz = self.xyz.ctypes.data_as(fp)
        c.features = self.features.ctypes.data_as(fp) if self.features is not None else fp()
        c.labels = self.labels.ctypes.data_as(fp) if self.labels is not None else fp()
        c.geom_type = self.geom_type.ctypes.data_as(fp) if self.geom_type is not None else fp()
        return c

    def transform(self, T: np.ndarray) -> "CvoPointCloud":
        """New cloud with positions mapped by the 4x4 transform T (CvoPointCloud::transform, :1529-1558)."""
        T = np.asarray(T, dtype=np.float64)
        p = (self.xyz.astype(np.float64) @ T[:3, :3].T + T[:3, 3]).astype(np.float32)
        return CvoPointCloud(p, self.features, self.labels, self.geom_type)

    def subset(self, idx) -> "CvoPointCloud":
        idx = np.asarray(idx)
        return CvoPointCloud(self.xyz[idx], None if self.features is None else self.features[idx],
                             None if self.labels is None else self.labels[idx],
                             None if self.geom_type is None else self.geom_type[idx])

    # -- file formats ---------------------------------------------------
    @staticmethod
    def read_pcd(path: str) -> "CvoPointCloud":
        """PCD v0.7 (ascii or binary).  x y z [rgb|rgba] [normal_x normal_y normal_z ...].

        With colour the cloud follows the pcl::PointXYZRGB constructor
        (src/utils/CvoPointCloud.cpp:576-604): features = (b, g, r) / 255 and
        geometric type (0, 1).  Without colour it has no features (XYZ / PointNormal
        constructors, :643-661, :673-694)."""
        with open(path, "rb") as fh:
            raw = fh.read()
        header = {}
        pos = 0
        while True:
            end = raw.index(b"\n", pos)
            line = raw[pos:end].decode("ascii", "replace").strip()
            pos = end + 1
            if not line or line.startswith("#"):
                continue
            key, _, val = line.partition(" ")
            header[key.upper()] = val.split()
            if key.upper() == "DATA":
                break
        fields = header["FIELDS"]
        sizes = [int(s) for s in header["SIZE"]]
        types = header["TYPE"]
        counts = [int(c) for c in header.get("COUNT", ["1"] * len(fields))]
        npts = int(header["POINTS"][0])
        mode = header["DATA"][0].lower()
        cols = {}
        if mode == "ascii":
            txt = raw[pos:].decode("ascii").split()
            ncol = sum(counts)
            vals = np.array(txt[: npts * ncol], dtype=np.float64).reshape(npts, ncol)
            k = 0
            for f, c, t in zip(fields, counts, types):
                cols[f] = vals[:, k:k + c]
                if t == "U" and f in ("rgb", "rgba"):
                    cols[f] = vals[:, k:k + c].astype(np.uint64).astype(np.uint32)
                k += c
        elif mode == "binary":
            dt = []
            for f, s, t, c in zip(fields, sizes, types, counts):
                base = {"F": {4: "<f4", 8: "<f8"}, "U": {1: "u1", 2: "<u2", 4: "<u4"}, "I": {1: "i1", 2: "<i2", 4: "<i4"}}[t][s]
                dt.append((f if f != "_" else "pad%d" % len(dt), base, (c,)))
            arr = np.frombuffer(raw, dtype=np.dtype(dt), count=npts, offset=pos)
            for f, _, _ in dt:
                cols[f] = np.asarray(arr[f]).reshape(npts, -1)
        else:
            raise ValueError("unsupported PCD DATA mode: %s" % mode)
        xyz = np.concatenate([cols["x"], cols["y"], cols["z"]], axis=1).astype(np.float32)
        feats = geo = None
        rgbkey = "rgb" if "rgb" in cols else ("rgba" if "rgba" in cols else None)
        if rgbkey:
            v = cols[rgbkey][:, 0]
            if v.dtype != np.uint32:
                v = np.asarray(v, np.float32).view(np.uint32)
            r = ((v >> 16) & 0xFF).astype(np.float32)
            g = ((v >> 8) & 0xFF).astype(np.float32)
            b = (v & 0xFF).astype(np.float32)
            feats = np.stack([b / 255.0, g / 255.0, r / 255.0], axis=1).astype(np.float32)
            geo = np.tile(np.array([[0.0, 1.0]], np.float32), (npts, 1))
        return CvoPointCloud(xyz, feats, None, geo)

    @staticmethod
    def read_txt(path: str) -> "CvoPointCloud":
        """read_cvo_pointcloud_from_file (src/utils/CvoPointCloud.cpp:1230-1273):
        header "N F C", then per point "u v idepth f_1..f_F x y z l_1..l_C"."""
        with open(path) as fh:
            tok = fh.read().split()
        n, F, Cc = int(tok[0]), int(tok[1]), int(tok[2])
        vals = np.array(tok[3: 3 + n * (3 + F + 3 + Cc)], dtype=np.float32).reshape(n, 3 + F + 3 + Cc)
        feats = vals[:, 3:3 + F] if F else None
        xyz = vals[:, 3 + F:6 + F]
        labels = vals[:, 6 + F:] if Cc else None
        return CvoPointCloud(xyz, feats, labels)

    def write_txt(self, path: str) -> None:
        """write_to_txt (src/utils/CvoPointCloud.cpp:1488-1510): "N C", then per point
        a line "x y z" and a line with the features and labels."""
        with open(path, "w") as fh:
            fh.write("%d %d\n" % (self.num_points(), self.num_classes()))
            for i in range(self.num_points()):
                fh.write("%g %g %g\n" % tuple(self.xyz[i]))
                parts = []
                if self.features is not None:
                    parts += ["%g" % v for v in self.features[i]]
                if self.labels is not None:
                    parts += ["%g" % v for v in self.labels[i]]
                fh.write(" ".join(parts) + " \n")

    def write_pcd(self, path: str) -> None:
        """Binary PCD with x y z (+ rgb when the cloud has >= 3 features, stored as b, g, r)."""
        n = self.num_points()
        has_rgb = self.features is not None and self.features.shape[1] >= 3
        fields = "x y z rgb" if has_rgb else "x y z"
        hdr = ("# .PCD v0.7 - Point Cloud Data file format\nVERSION 0.7\nFIELDS %s\nSIZE %s\nTYPE %s\nCOUNT %s\n"
               "WIDTH %d\nHEIGHT 1\nVIEWPOINT 0 0 0 1 0 0 0\nPOINTS %d\nDATA binary\n" %
               (fields, " ".join(["4"] * (4 if has_rgb else 3)), "F F F U" if has_rgb else "F F F",
                " ".join(["1"] * (4 if has_rgb else 3)), n, n))
        if has_rgb:
            f = np.clip(np.round(self.features[:, :3] * 255.0), 0, 255).astype(np.uint32)
            rgb = (f[:, 2] << 16) | (f[:, 1] << 8) | f[:, 0]
            rec = np.zeros(n, dtype=[("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("rgb", "<u4")])
            rec["rgb"] = rgb
        else:
            rec = np.zeros(n, dtype=[("x", "<f4"), ("y", "<f4"), ("z", "<f4")])
        rec["x"], rec["y"], rec["z"] = self.xyz[:, 0], self.xyz[:, 1], self.xyz[:, 2]
        with open(path, "wb") as fh:
            fh.write(hdr.encode("ascii"))
            fh.write(rec.tobytes())

