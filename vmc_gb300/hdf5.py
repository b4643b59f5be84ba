"""Minimal read-only HDF5 reader for the reference's ``FCIDUMP_chol`` files.

The reference writes its Cholesky integral files with h5py
(scripts/QMCUtils.py:1067-1097) and reads them with libhdf5 in
utils/integral.cpp:589-741 (datasets ``header``, ``hcore``, ``hcore_mod``,
``chol``, ``energy_core``; the ``intType: "u"`` variant has ``*_up``/``*_dn``).
Neither libhdf5 nor h5py is a dependency here, so this module implements the
small subset of the public HDF5 file-format specification that such files use:

* superblock version 0 or 1 (symbol-table root group),
* version-1 B-trees of group nodes with ``SNOD`` symbol-table nodes and a local heap,
* version-1 object headers (with continuation blocks),
* dataspace (0x0001), datatype (0x0003, fixed-point or IEEE float, little endian),
  and data-layout (0x0008: compact or contiguous) messages.

Chunked or filtered datasets raise ``NotImplementedError``.
"""
import struct

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"


class H5File:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.buf = f.read()
        if self.buf[:8] != _SIG:
            raise ValueError(f"{path}: not an HDF5 file")
        ver = self.buf[8]
        if ver not in (0, 1):
            raise NotImplementedError(f"superblock version {ver}")
        self.so = self.buf[13]  # size of offsets
        self.sl = self.buf[14]  # size of lengths
        pos = 24 + (4 if ver == 1 else 0)
        pos += 4 * self.so  # base, free-space, EOF, driver addresses
        # root group symbol table entry
        _, self.root_ohdr, ctype = self._entry(pos)
        self.datasets = {}
        self._walk_group(self.root_ohdr, "")

    # --- primitive readers -------------------------------------------------
    def _u(self, pos, n):
        return int.from_bytes(self.buf[pos:pos + n], "little")

    def _entry(self, pos):
        name_off = self._u(pos, self.so)
        ohdr = self._u(pos + self.so, self.so)
        ctype = self._u(pos + 2 * self.so, 4)
        return name_off, ohdr, ctype

    def _heap_data(self, addr):
        if self.buf[addr:addr + 4] != b"HEAP":
            raise ValueError("bad local heap")
        p = addr + 8 + 2 * self.sl
        return self._u(p, self.so)

    def _cstr(self, pos):
        end = self.buf.index(b"\x00", pos)
        return self.buf[pos:end].decode()

    # --- object headers ----------------------------------------------------
    def _messages(self, addr):
        if self.buf[addr] != 1:
            raise NotImplementedError(f"object header version {self.buf[addr]}")
        nmsg = self._u(addr + 2, 2)
        size = self._u(addr + 8, 4)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p = start
            while p + 8 <= start + length and len(out) < nmsg:
                mtype = self._u(p, 2)
                msize = self._u(p + 2, 2)
                data = p + 8
                if mtype == 0x0010:  # continuation
                    blocks.append((self._u(data, self.so), self._u(data + self.so, self.sl)))
                out.append((mtype, data, msize))
                p = data + msize
        return out

    def _walk_group(self, ohdr, prefix):
        btree = heap = None
        for mtype, data, _ in self._messages(ohdr):
            if mtype == 0x0011:  # symbol table message
                btree = self._u(data, self.so)
                heap = self._u(data + self.so, self.so)
        if btree is None:
            raise NotImplementedError("only symbol-table groups are supported")
        heap_data = self._heap_data(heap)
        for name_off, child in self._btree_entries(btree):
            name = self._cstr(heap_data + name_off)
            path = prefix + "/" + name
            kinds = {m[0] for m in self._messages(child)}
            if 0x0011 in kinds:
                self._walk_group(child, path)
            else:
                self.datasets[path] = child

    def _btree_entries(self, addr):
        if self.buf[addr:addr + 4] != b"TREE":
            raise ValueError("bad B-tree node")
        level = self.buf[addr + 5]
        used = self._u(addr + 6, 2)
        p = addr + 8 + 2 * self.so + self.sl  # skip siblings and key 0
        for _ in range(used):
            child = self._u(p, self.so)
            p += self.so + self.sl
            if level > 0:
                yield from self._btree_entries(child)
            else:
                yield from self._snod_entries(child)

    def _snod_entries(self, addr):
        if self.buf[addr:addr + 4] != b"SNOD":
            raise ValueError("bad symbol table node")
        nsym = self._u(addr + 6, 2)
        esize = 2 * self.so + 8 + 16
        for i in range(nsym):
            name_off, ohdr, _ = self._entry(addr + 8 + i * esize)
            yield name_off, ohdr

    # --- datasets ----------------------------------------------------------
    def keys(self):
        return sorted(k.lstrip("/") for k in self.datasets)

    def __contains__(self, name):
        return ("/" + name.lstrip("/")) in self.datasets

    def read(self, name):
        ohdr = self.datasets["/" + name.lstrip("/")]
        shape = dtype = None
        raw = None
        for mtype, data, msize in self._messages(ohdr):
            if mtype == 0x0001:
                shape = self._dataspace(data)
            elif mtype == 0x0003:
                dtype = self._datatype(data)
            elif mtype == 0x0008:
                raw = self._layout(data)
            elif mtype == 0x000B:
                raise NotImplementedError("filtered datasets are not supported")
        count = int(np.prod(shape)) if shape else 1
        nbytes = count * dtype.itemsize
        if raw[0] == "compact":
            blob = self.buf[raw[1]:raw[1] + nbytes]
        else:
            blob = self.buf[raw[1]:raw[1] + nbytes]
        arr = np.frombuffer(blob, dtype=dtype, count=count).copy()
        return arr.reshape(shape) if shape else arr.reshape(())

    def _dataspace(self, p):
        ver = self.buf[p]
        ndim = self.buf[p + 1]
        q = p + (8 if ver == 1 else 4)
        return tuple(self._u(q + i * self.sl, self.sl) for i in range(ndim))

    def _datatype(self, p):
        cls = self.buf[p] & 0x0F
        bits = self.buf[p + 1]
        size = self._u(p + 4, 4)
        if bits & 1:
            raise NotImplementedError("big-endian data")
        if cls == 0:
            signed = bool(bits & 0x08)
            return np.dtype(("<i" if signed else "<u") + str(size))
        if cls == 1:
            return np.dtype("<f" + str(size))
        raise NotImplementedError(f"datatype class {cls}")

    def _layout(self, p):
        ver = self.buf[p]
        if ver == 3:
            cls = self.buf[p + 1]
            if cls == 0:
                return ("compact", p + 4)
            if cls == 1:
                return ("contiguous", self._u(p + 2, self.so))
            raise NotImplementedError("chunked datasets are not supported")
        if ver in (1, 2):
            ndim = self.buf[p + 1]
            cls = self.buf[p + 2]
            q = p + 8
            if cls == 0:
                q += 4 * ndim
                return ("compact", q + 4)
            if cls == 1:
                return ("contiguous", self._u(q, self.so))
            raise NotImplementedError("chunked datasets are not supported")
        raise NotImplementedError(f"layout message version {ver}")


def read_fcidump_chol(path):
    """Return the DQMC integral file as a dict, following the dataset names that
    utils/integral.cpp:589-661 (restricted) and :664-741 (``_up``/``_dn``) read."""
    f = H5File(path)
    out = {"keys": f.keys()}
    hdr = f.read("header").astype(np.int64).ravel()
    nelec, norb, ms, nchol = (int(v) for v in hdr[:4])
    out.update(nelec=nelec, norb=norb, ms=ms, nchol=nchol)
    out["nalpha"] = (nelec + ms) // 2
    out["nbeta"] = nelec - out["nalpha"]
    out["ecore"] = float(f.read("energy_core").ravel()[0]) if "energy_core" in f else 0.0
    if "hcore" in f:
        out["h1"] = f.read("hcore").reshape(norb, norb)
        out["h1mod"] = f.read("hcore_mod").reshape(norb, norb)
        out["chol"] = f.read("chol").reshape(nchol, norb, norb)
    else:
        out["h1u"] = np.stack([f.read("hcore_up").reshape(norb, norb),
                               f.read("hcore_dn").reshape(norb, norb)])
        out["h1umod"] = np.stack([f.read("hcore_mod_up").reshape(norb, norb),
                                  f.read("hcore_mod_dn").reshape(norb, norb)])
        out["cholu"] = np.stack([f.read("chol_up").reshape(nchol, norb, norb),
                                 f.read("chol_dn").reshape(nchol, norb, norb)])
    return out
