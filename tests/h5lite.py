"""A small pure-Python HDF5 decoder for the structures samurai's files use
(superblock version 0, version 1 object headers, symbol-table groups with
version 1 B-trees and local heaps, contiguous or compact datasets of integers,
binary64 floats or compound types).  h5py is not available here; the tests
use this decoder as an independent check of the files the library writes and
the golden-fixture script uses it to read the reference's own files.
"""
import struct

import numpy as np


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
            node = stack.pop(0)
            assert self.b[node:node + 4] == b"TREE"
            ntype, level, used = struct.unpack_from("<BBH", self.b, node + 4)
            assert ntype == 0
            p = node + 8 + 16 + 8  # header, siblings, key0
            children = []
            for _ in range(used):
                children.append(self.u64(p))
                p += 16
            if level > 0:
                stack = children + stack
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

    def dtype_at(self, data):
        """numpy dtype of a datatype message body; returns (dtype, bytes used)"""
        cls = self.b[data] & 0x0F
        ver = self.b[data] >> 4
        bits = self.b[data + 1]
        size = struct.unpack_from("<I", self.b, data + 4)[0]
        if cls == 1:
            return np.dtype({8: "<f8", 4: "<f4"}[size]), 8 + 12
        if cls == 0:
            signed = bool(bits & 0x08)
            return np.dtype(("<i" if signed else "<u") + str(size)), 8 + 4
        if cls == 6:
            nmem = struct.unpack_from("<H", self.b, data + 1)[0]
            p = data + 8
            names, offsets, types = [], [], []
            for _ in range(nmem):
                end = self.b.index(b"\0", p)
                name = self.b[p:end].decode()
                if ver == 3:
                    p = end + 1
                    nb = 1 if size < 256 else 2 if size < 65536 else 3 if size < (1 << 24) else 4
                    off = int.from_bytes(self.b[p:p + nb], "little")
                    p += nb
                else:
                    p += (len(name) + 1 + 7) // 8 * 8
                    off = struct.unpack_from("<I", self.b, p)[0]
                    p += 32 if ver == 1 else 4
                mt, used = self.dtype_at(p)
                p += used
                names.append(name)
                offsets.append(off)
                types.append(mt)
            return np.dtype({"names": names, "formats": types, "offsets": offsets, "itemsize": size}), p - data
        raise ValueError("unsupported datatype class %d" % cls)

    def dataset(self, ohdr):
        shape = dtype = addr = None
        for mtype, data, msize in self.messages(ohdr):
            if mtype == 0x0001:
                ver = self.b[data]
                nd = self.b[data + 1]
                p = data + (8 if ver == 1 else 4)
                shape = tuple(self.u64(p + 8 * k) for k in range(nd))
            elif mtype == 0x0003:
                dtype = self.dtype_at(data)[0]
            elif mtype == 0x0008:
                ver = self.b[data]
                if ver == 3:
                    cls = self.b[data + 1]
                    assert cls in (0, 1), "only contiguous and compact layouts are decoded"
                    addr = self.u64(data + 2) if cls == 1 else data + 4
                else:
                    cls = self.b[data + 2]
                    assert cls == 1
                    addr = self.u64(data + 8)
            elif mtype == 0x000B:
                raise ValueError("filtered datasets are not decoded")
        n = int(np.prod(shape)) if shape else 1
        if n == 0:
            return np.zeros(shape, dtype)
        arr = np.frombuffer(self.b, dtype=dtype, count=n, offset=addr)
        return arr.reshape(shape)

    def _walk(self, path):
        cur = self.group_entries(*self.root)
        parts = [p for p in path.strip("/").split("/") if p]
        entry = None
        for k, name in enumerate(parts):
            entry = cur[name]
            if k < len(parts) - 1:
                cur = self.group(*entry)
        return entry, cur

    def read(self, path):
        (ohdr, _), _ = self._walk(path)
        return self.dataset(ohdr)

    def exists(self, path):
        try:
            self._walk(path)
            return True
        except KeyError:
            return False

    def keys(self, path="/"):
        """member names of a group, in the order the file stores them"""
        if path.strip("/") == "":
            return list(self.group_entries(*self.root).keys())
        entry, _ = self._walk(path)
        return list(self.group(*entry).keys())
