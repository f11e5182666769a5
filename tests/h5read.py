"""A small HDF5 reader for the snapshot tests (test infrastructure only).

h5py and libhdf5 are not available here, so the snapshot files are read with this
parser of the published HDF5 file format: superblock version 0 or 1, groups stored as
symbol tables (version-1 B-tree + symbol table nodes + local heap), version-1 object
headers, and contiguous datasets of IEEE floating-point numbers. It is checked against
a file written by libhdf5 itself (a MATLAB 7.3 test file that SciPy ships, where
present), then used to read the files the library writes.
"""
from __future__ import annotations

import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(ValueError):
    pass


class File:
    def __init__(self, path: str):
        with open(path, "rb") as fh:
            self.raw = fh.read()
        base = None
        for off in (0, 512, 1024, 2048, 4096, 8192):
            if self.raw[off:off + 8] == SIG:
                base = off
                break
        if base is None:
            raise H5Error("no HDF5 signature")
        self.base = base
        r = self.raw
        sb_ver = r[base + 8]
        if sb_ver not in (0, 1):
            raise H5Error(f"superblock version {sb_ver} not supported")
        self.so, self.sl = r[base + 13], r[base + 14]
        if (self.so, self.sl) != (8, 8):
            raise H5Error("only 8-byte offsets and lengths")
        self.leaf_k, self.int_k = struct.unpack_from("<HH", r, base + 16)
        p = base + 24 + (4 if sb_ver == 1 else 0)
        self.base_addr, self.free_addr, self.eof, self.driver = struct.unpack_from("<4Q", r, p)
        self.root_entry = self._entry(p + 32)
        if self.root_entry["cache"] != 1:
            raise H5Error("root entry without cached symbol table")
        self.root = self._group(self.root_entry["ohdr"])
        if (self.root_entry["btree"], self.root_entry["heap"]) != self.root["stab"]:
            raise H5Error("root entry scratch pad disagrees with the symbol table message")

    # --------------------------------------------------------------- low level
    def _abs(self, addr: int) -> int:
        a = self.base + addr
        if addr == UNDEF or a > len(self.raw):
            raise H5Error(f"address {addr:#x} outside the file")
        return a

    def _entry(self, p: int) -> dict:
        name_off, ohdr, cache = struct.unpack_from("<QQI", self.raw, p)
        e = {"name_off": name_off, "ohdr": ohdr, "cache": cache}
        if cache == 1:
            e["btree"], e["heap"] = struct.unpack_from("<QQ", self.raw, p + 24)
        return e

    def _messages(self, addr: int) -> list:
        r, p = self.raw, self._abs(addr)
        ver, nmsg, refcnt, size = r[p], *struct.unpack_from("<HII", r, p + 2)
        if ver != 1:
            raise H5Error(f"object header version {ver} not supported")
        msgs, chunks = [], [(p + 16, size)]
        while chunks:
            q, sz = chunks.pop(0)
            end = q + sz
            while q + 8 <= end:
                mtype, msize, flags = struct.unpack_from("<HHB", r, q)
                if q + 8 + msize > end:
                    raise H5Error("message runs past its chunk")
                body = r[q + 8:q + 8 + msize]
                if mtype == 0x10:   # continuation
                    caddr, clen = struct.unpack_from("<QQ", body, 0)
                    chunks.append((self._abs(caddr), clen))
                msgs.append((mtype, flags, body))
                q += 8 + msize
        if len(msgs) != nmsg:
            raise H5Error(f"object header lists {nmsg} messages, found {len(msgs)}")
        return msgs

    def _heap(self, addr: int):
        r, p = self.raw, self._abs(addr)
        if r[p:p + 4] != b"HEAP":
            raise H5Error("bad local heap signature")
        size, free_head, data = struct.unpack_from("<QQQ", r, p + 8)
        seg = r[self._abs(data):self._abs(data) + size]
        if len(seg) != size:
            raise H5Error("local heap data segment truncated")
        fb = free_head
        while fb != 1:    # 1 ends the free list
            if fb >= size:
                raise H5Error("bad local heap free list")
            nxt, fsz = struct.unpack_from("<QQ", seg, fb)
            if fsz < 16 or fb + fsz > size:
                raise H5Error("bad local heap free block")
            fb = nxt
        return seg

    @staticmethod
    def _name(seg: bytes, off: int) -> str:
        end = seg.index(b"\0", off)
        return seg[off:end].decode()

    def _group(self, addr: int) -> dict:
        stab = None
        for mtype, _, body in self._messages(addr):
            if mtype == 0x11:
                stab = struct.unpack_from("<QQ", body, 0)
        if stab is None:
            raise H5Error("group without a symbol table message")
        seg = self._heap(stab[1])
        links = {}
        self._walk(stab[0], seg, links)
        names = list(links)
        if names != sorted(names):
            raise H5Error("symbol table entries not sorted by name")
        return {"stab": stab, "links": links}

    def _walk(self, addr: int, seg: bytes, links: dict) -> None:
        r, p = self.raw, self._abs(addr)
        if r[p:p + 4] != b"TREE":
            raise H5Error("bad B-tree signature")
        ntype, level, used = r[p + 4], r[p + 5], struct.unpack_from("<H", r, p + 6)[0]
        if ntype != 0:
            raise H5Error("not a group B-tree")
        if used > 2 * self.int_k:
            raise H5Error("B-tree node over-full")
        q = p + 24
        keys, children = [struct.unpack_from("<Q", r, q)[0]], []
        q += 8
        for _ in range(used):
            c, k = struct.unpack_from("<QQ", r, q)
            children.append(c)
            keys.append(k)
            q += 16
        for i, c in enumerate(children):
            if level > 0:
                self._walk(c, seg, links)
                continue
            s = self._abs(c)
            if r[s:s + 4] != b"SNOD" or r[s + 4] != 1:
                raise H5Error("bad symbol table node")
            nsym = struct.unpack_from("<H", r, s + 6)[0]
            if nsym > 2 * self.leaf_k:
                raise H5Error("symbol table node over-full")
            last = None
            for e in range(nsym):
                ent = self._entry(s + 8 + 40 * e)
                last = self._name(seg, ent["name_off"])
                links[last] = ent["ohdr"]
            if last is not None and self._name(seg, keys[i + 1]) != last:
                raise H5Error("B-tree key is not the child's last name")

    # --------------------------------------------------------------- datasets
    def keys(self) -> list:
        return list(self.root["links"])

    def dataset_info(self, name: str) -> dict:
        name = name.lstrip("/")
        addr = self.root["links"][name]
        info = {}
        for mtype, _, b in self._messages(addr):
            if mtype == 0x0001:
                ver, rank, flags = b[0], b[1], b[2]
                off = 8 if ver == 1 else 4
                info["shape"] = tuple(struct.unpack_from(f"<{rank}Q", b, off))
            elif mtype == 0x0003:
                cls, ver = b[0] & 0x0F, b[0] >> 4
                size = struct.unpack_from("<I", b, 4)[0]
                if cls != 1:
                    raise H5Error(f"datatype class {cls} is not floating point")
                big = b[1] & 1
                _, prec, eloc, esz, mloc, msz, bias = struct.unpack_from("<HHBBBBI", b, 8)
                if size == 8 and (prec, eloc, esz, mloc, msz, bias) != (64, 52, 11, 0, 52, 1023):
                    raise H5Error("8-byte float that is not IEEE binary64")
                info["dtype"] = np.dtype((">" if big else "<") + f"f{size}")
                info["type_bits"] = bytes(b[1:4])
            elif mtype == 0x0008:
                ver = b[0]
                if ver == 3:
                    if b[1] != 1:
                        raise H5Error("only contiguous layout")
                    info["addr"], info["nbytes"] = struct.unpack_from("<QQ", b, 2)
                elif ver in (1, 2):
                    ndim, cls = b[1], b[2]
                    if cls != 1:
                        raise H5Error("only contiguous layout")
                    info["addr"] = struct.unpack_from("<Q", b, 8)[0]
                    dims = struct.unpack_from(f"<{ndim}I", b, 16)
                    info["nbytes"] = int(np.prod(dims, dtype=np.int64))
                else:
                    raise H5Error(f"layout version {ver}")
            elif mtype == 0x0005:
                info["fill"] = bytes(b)
        for k in ("shape", "dtype", "addr", "nbytes"):
            if k not in info:
                raise H5Error(f"dataset {name} lacks its {k}")
        return info

    def read(self, name: str) -> np.ndarray:
        info = self.dataset_info(name)
        count = int(np.prod(info["shape"], dtype=np.int64))
        if count * info["dtype"].itemsize != info["nbytes"]:
            raise H5Error("layout size disagrees with dataspace x datatype")
        p = self._abs(info["addr"])
        if p + info["nbytes"] > len(self.raw) or info["addr"] + info["nbytes"] > self.eof:
            raise H5Error("dataset extends past the end of file")
        return np.frombuffer(self.raw, dtype=info["dtype"], count=count, offset=p).reshape(info["shape"])
