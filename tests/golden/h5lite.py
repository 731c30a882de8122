"""Minimal read-only HDF5 reader for the reference's golden files.

Test infrastructure only: it is used by ``make_fixtures.py`` to turn the
reference's HDF5 goldens (written by HighFive / libhdf5 1.x defaults) into
small ``.npz`` fixtures.  No h5py or libhdf5 exists in this environment, so
this module parses the on-disk format directly.

Supported subset (all that the goldens use):
  * superblock version 0/1, object headers version 1 (with continuation),
  * old-style groups (symbol table message, v1 group B-tree, SNOD, local heap),
  * dataspace messages v1/v2,
  * datatypes: fixed-point, floating-point, compound (v1-v3), array,
  * data layout message v3: compact and contiguous (no chunking/filters).
"""
import struct
import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class H5File:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.buf = f.read()
        b = self.buf
        if b[:8] != b"\x89HDF\r\n\x1a\n":
            raise ValueError("not an HDF5 file")
        ver = b[8]
        if ver not in (0, 1):
            raise ValueError(f"unsupported superblock version {ver}")
        self.so = b[13]
        self.sl = b[14]
        assert self.so == 8 and self.sl == 8
        off = 24 if ver == 0 else 28
        off += 4 * 8  # base, freespace, eof, driver
        # root symbol table entry
        _, ohdr = struct.unpack_from("<QQ", b, off)
        self.root = ohdr

    # ---------------------------------------------------------------- objects
    def _messages(self, addr):
        b = self.buf
        ver = b[addr]
        if ver != 1:
            raise ValueError(f"object header version {ver} unsupported")
        nmsg, = struct.unpack_from("<H", b, addr + 2)
        hsize, = struct.unpack_from("<I", b, addr + 8)
        blocks = [(addr + 16, hsize)]
        msgs = []
        while blocks and len(msgs) < nmsg:
            start, size = blocks.pop(0)
            p = start
            while p + 8 <= start + size and len(msgs) < nmsg:
                mtype, msize, mflags = struct.unpack_from("<HHB", b, p)
                data_off = p + 8
                if mtype == 0x10:  # continuation
                    caddr, clen = struct.unpack_from("<QQ", b, data_off)
                    blocks.append((caddr, clen))
                msgs.append((mtype, data_off, msize))
                p = data_off + msize
        return msgs

    def _group_links(self, addr):
        """Return {name: object_header_address} for an old-style group."""
        for mtype, off, _ in self._messages(addr):
            if mtype == 0x11:
                btree, heap = struct.unpack_from("<QQ", self.buf, off)
                return self._walk_group_btree(btree, heap)
        raise ValueError("object is not a (symbol-table) group")

    def _heap_data(self, heap):
        b = self.buf
        assert b[heap:heap + 4] == b"HEAP"
        _, _, daddr = struct.unpack_from("<QQQ", b, heap + 8)
        return daddr

    def _walk_group_btree(self, btree, heap):
        b = self.buf
        daddr = self._heap_data(heap)
        out = {}

        def name_at(o):
            e = b.index(b"\x00", daddr + o)
            return b[daddr + o:e].decode()

        def walk(node):
            assert b[node:node + 4] == b"TREE", "bad btree node"
            ntype, level, nused = struct.unpack_from("<BBH", b, node + 4)
            assert ntype == 0
            p = node + 8 + 16
            children = []
            for i in range(nused):
                p += 8  # key
                child, = struct.unpack_from("<Q", b, p)
                p += 8
                children.append(child)
            for c in children:
                if level > 0:
                    walk(c)
                else:
                    assert b[c:c + 4] == b"SNOD"
                    nsym, = struct.unpack_from("<H", b, c + 6)
                    q = c + 8
                    for _ in range(nsym):
                        lno, oh = struct.unpack_from("<QQ", b, q)
                        out[name_at(lno)] = oh
                        q += 40

        walk(btree)
        return out

    # ---------------------------------------------------------------- lookup
    def _resolve(self, path):
        addr = self.root
        for part in [p for p in path.split("/") if p]:
            links = self._group_links(addr)
            if part not in links:
                raise KeyError(path)
            addr = links[part]
        return addr

    def exists(self, path):
        try:
            self._resolve(path)
            return True
        except KeyError:
            return False

    def keys(self, path="/"):
        return sorted(self._group_links(self._resolve(path)).keys())

    # ---------------------------------------------------------------- datasets
    def _parse_dtype(self, off):
        b = self.buf
        cv = b[off]
        cls = cv & 0x0F
        ver = cv >> 4
        bits = b[off + 1] | (b[off + 2] << 8) | (b[off + 3] << 16)
        size, = struct.unpack_from("<I", b, off + 4)
        p = off + 8
        if cls == 0:  # fixed point
            assert (bits & 1) == 0, "big endian unsupported"
            signed = bool(bits & 0x08)
            dt = np.dtype(("<i" if signed else "<u") + str(size))
            return dt, p + 4
        if cls == 1:  # float
            assert (bits & 1) == 0
            dt = np.dtype("<f" + str(size))
            return dt, p + 12
        if cls == 6:  # compound
            nmemb = bits & 0xFFFF
            names, formats, offsets = [], [], []
            for _ in range(nmemb):
                e = b.index(b"\x00", p)
                name = b[p:e].decode()
                if ver < 3:
                    nlen = e - p + 1
                    p += (nlen + 7) // 8 * 8
                else:
                    p = e + 1
                if ver == 1:
                    moff, = struct.unpack_from("<I", b, p)
                    ndim = b[p + 4]
                    p += 4 + 1 + 3 + 4 + 4
                    dims = struct.unpack_from("<4I", b, p)[:ndim]
                    p += 16
                    mdt, p = self._parse_dtype(p)
                    if ndim:
                        mdt = np.dtype((mdt, tuple(dims)))
                elif ver == 2:
                    moff, = struct.unpack_from("<I", b, p)
                    p += 4
                    mdt, p = self._parse_dtype(p)
                else:
                    nb = 1 if size < 256 else 2 if size < 65536 else 3 if size < (1 << 24) else 4
                    moff = int.from_bytes(b[p:p + nb], "little")
                    p += nb
                    mdt, p = self._parse_dtype(p)
                names.append(name)
                formats.append(mdt)
                offsets.append(moff)
            dt = np.dtype({"names": names, "formats": formats,
                           "offsets": offsets, "itemsize": size})
            return dt, p
        if cls == 10:  # array
            ndim = b[p]
            if ver == 2:
                p += 4
                dims = struct.unpack_from("<%dI" % ndim, b, p)
                p += 4 * ndim + 4 * ndim
            else:
                p += 1
                dims = struct.unpack_from("<%dI" % ndim, b, p)
                p += 4 * ndim
            base, p = self._parse_dtype(p)
            return np.dtype((base, tuple(dims))), p
        raise ValueError(f"datatype class {cls} unsupported")

    def read(self, path):
        addr = self._resolve(path)
        b = self.buf
        shape = None
        dtype = None
        data = None
        for mtype, off, msize in self._messages(addr):
            if mtype == 0x01:
                ver = b[off]
                ndim = b[off + 1]
                if ver == 1:
                    dims = struct.unpack_from("<%dQ" % ndim, b, off + 8)
                else:
                    dims = struct.unpack_from("<%dQ" % ndim, b, off + 4)
                shape = tuple(dims)
            elif mtype == 0x03:
                dtype, _ = self._parse_dtype(off)
            elif mtype == 0x08:
                ver = b[off]
                if ver != 3:
                    raise ValueError("layout version unsupported")
                lcls = b[off + 1]
                if lcls == 0:
                    n, = struct.unpack_from("<H", b, off + 2)
                    data = b[off + 4:off + 4 + n]
                elif lcls == 1:
                    a, n = struct.unpack_from("<QQ", b, off + 2)
                    data = b"" if a == UNDEF else b[a:a + n]
                else:
                    raise ValueError("chunked layout unsupported")
        if dtype is None or shape is None:
            raise ValueError(f"{path} is not a dataset")
        count = int(np.prod(shape)) if shape else 1
        if data is None or len(data) == 0:
            arr = np.zeros(count, dtype=dtype)
        else:
            arr = np.frombuffer(data, dtype=dtype, count=count)
        return arr.reshape(shape).copy()
