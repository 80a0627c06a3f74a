"""Convert the reference's committed advection_2d golden HDF5 outputs into
small .npz fixtures (level, i, j, u per leaf cell, in the files' cell order).

The reference's own pytest compares these files dataset by dataset
(tests/conftest.py:26-194 of hpc-maths/samurai); they are produced by
demos/FiniteVolume/advection_2d.cpp run with --Tf 0.01
(tests/test_demo_finite_volume.py:55-72).  h5py is not available here, so the
few HDF5 structures those files use (superblock v0, v1 object headers, v1
B-tree group nodes, local heaps, contiguous layout) are decoded by hand.

Run once in a container where the reference tree is mounted:
    python tests/golden/make_golden.py /root/reference
"""
import os
import struct
import sys

import numpy as np

NAMES = [
    "test_finite_volume_advection_2d_finite-volume-advection-2d-0.01_pred_0_init",
    "test_finite_volume_advection_2d_finite-volume-advection-2d-0.01_pred_0",
    "test_finite_volume_advection_2d_finite-volume-advection-2d-0.01_pred_1_init",
    "test_finite_volume_advection_2d_finite-volume-advection-2d-0.01_pred_1",
]


class H5:
    def __init__(self, path):
        self.b = open(path, "rb").read()
        assert self.b[:8] == b"\x89HDF\r\n\x1a\n", "not an HDF5 file"
        assert self.b[8] == 0, "only superblock version 0 is decoded"
        self.so = self.b[13]
        self.sl = self.b[14]
        assert self.so == 8 and self.sl == 8
        # root group symbol table entry at offset 56
        ent = 24 + 4 * 8
        cache = struct.unpack_from("<I", self.b, ent + 16)[0]
        assert cache == 1
        self.root = struct.unpack_from("<QQ", self.b, ent + 24)  # btree, heap

    def u64(self, off):
        return struct.unpack_from("<Q", self.b, off)[0]

    def heap_name(self, heap, off):
        assert self.b[heap:heap + 4] == b"HEAP"
        data = self.u64(heap + 24)
        end = self.b.index(b"\0", data + off)
        return self.b[data + off:end].decode()

    def group_entries(self, btree, heap):
        out = {}
        stack = [btree]
        while stack:
            node = stack.pop()
            assert self.b[node:node + 4] == b"TREE"
            ntype, level, used = struct.unpack_from("<BBH", self.b, node + 4)
            assert ntype == 0
            p = node + 8 + 16 + 8  # header, siblings, key0
            children = []
            for _ in range(used):
                children.append(self.u64(p))
                p += 16
            if level > 0:
                stack.extend(children)
                continue
            for snod in children:
                assert self.b[snod:snod + 4] == b"SNOD"
                nsym = struct.unpack_from("<H", self.b, snod + 6)[0]
                q = snod + 8
                for _ in range(nsym):
                    name_off, ohdr = struct.unpack_from("<QQ", self.b, q)
                    cache = struct.unpack_from("<I", self.b, q + 16)[0]
                    scratch = struct.unpack_from("<QQ", self.b, q + 24) if cache == 1 else None
                    out[self.heap_name(heap, name_off)] = (ohdr, scratch)
                    q += 40
        return out

    def messages(self, ohdr):
        assert self.b[ohdr] == 1, "only v1 object headers are decoded"
        nmsg = struct.unpack_from("<H", self.b, ohdr + 2)[0]
        size = struct.unpack_from("<I", self.b, ohdr + 8)[0]
        blocks = [(ohdr + 16, size)]
        msgs = []
        while blocks and len(msgs) < nmsg:
            start, length = blocks.pop(0)
            p = start
            while p < start + length and len(msgs) < nmsg:
                mtype, msize, flags = struct.unpack_from("<HHB", self.b, p)
                data = p + 8
                if mtype == 0x10:
                    blocks.append((self.u64(data), self.u64(data + 8)))
                msgs.append((mtype, data, msize))
                p = data + msize
        return msgs

    def group(self, ohdr, scratch):
        if scratch is not None:
            return self.group_entries(*scratch)
        for mtype, data, _ in self.messages(ohdr):
            if mtype == 0x11:
                return self.group_entries(self.u64(data), self.u64(data + 8))
        raise ValueError("object is not a group")

    def dataset(self, ohdr):
        shape = dtype = addr = None
        for mtype, data, msize in self.messages(ohdr):
            if mtype == 0x0001:
                ver = self.b[data]
                nd = self.b[data + 1]
                p = data + (8 if ver == 1 else 4)
                shape = tuple(self.u64(p + 8 * k) for k in range(nd))
            elif mtype == 0x0003:
                cls = self.b[data] & 0x0F
                bits = self.b[data + 1]
                size = struct.unpack_from("<I", self.b, data + 4)[0]
                if cls == 1:
                    dtype = {8: "<f8", 4: "<f4"}[size]
                elif cls == 0:
                    signed = bool(bits & 0x08)
                    dtype = ("<i" if signed else "<u") + str(size)
                else:
                    raise ValueError("unsupported datatype class %d" % cls)
            elif mtype == 0x0008:
                ver = self.b[data]
                if ver == 3:
                    cls = self.b[data + 1]
                    assert cls == 1, "only contiguous layout is decoded"
                    addr = self.u64(data + 2)
                else:
                    cls = self.b[data + 2]
                    assert cls == 1
                    addr = self.u64(data + 8)
            elif mtype == 0x000B:
                raise ValueError("filtered datasets are not decoded")
        n = int(np.prod(shape)) if shape else 1
        arr = np.frombuffer(self.b, dtype=dtype, count=n, offset=addr)
        return arr.reshape(shape)

    def read(self, path):
        node = (None, self.root)
        cur = self.group_entries(*self.root)
        parts = path.strip("/").split("/")
        for k, name in enumerate(parts):
            ohdr, scratch = cur[name]
            if k == len(parts) - 1:
                return self.dataset(ohdr)
            cur = self.group(ohdr, scratch)


def convert(src_dir, name, out_dir):
    h = H5(os.path.join(src_dir, name + ".h5"))
    pts = h.read("/mesh/points")
    conn = h.read("/mesh/connectivity").astype(np.int64)
    u = h.read("/mesh/fields/u").astype(np.float64)
    p0 = pts[conn[:, 0]]
    p2 = pts[conn[:, 2]]
    length = p2[:, 0] - p0[:, 0]
    level = np.rint(-np.log2(length)).astype(np.int8)
    scale = np.ldexp(1.0, level.astype(np.int64))
    i = np.rint(p0[:, 0] * scale).astype(np.int32)
    j = np.rint(p0[:, 1] * scale).astype(np.int32)
    # corners must be exact dyadic numbers
    assert np.all(i / scale == p0[:, 0]) and np.all(j / scale == p0[:, 1])
    np.savez_compressed(os.path.join(out_dir, name.split("2d-0.01_")[1] + ".npz"), level=level, i=i, j=j, u=u)
    return len(u)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    src = os.path.join(ref, "tests", "reference", "finite_volume")
    out = os.path.dirname(os.path.abspath(__file__))
    for name in NAMES:
        n = convert(src, name, out)
        print(name, n, "cells")


if __name__ == "__main__":
    main()
