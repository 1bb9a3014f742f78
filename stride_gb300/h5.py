"""Mosaic's HDF5 file layer (mosaic/file_manipulation/h5.py) without h5py.

Stride dumps and loads its problem objects (fields, traces, geometries) as HDF5 files through
``mosaic.file_manipulation.h5.HDF5``, which wraps h5py. Neither h5py nor libhdf5 is a dependency
here, so this module reads and writes the subset of the HDF5 file format (the public HDF Group
specification) that those files use:

* reading: superblocks v0 (libhdf5 defaults) and v2/v3 (``libver='latest'``, which mosaic opens
  with); object headers v1 and v2 with continuation blocks; groups as symbol tables (v1 B-tree,
  symbol-table nodes, local heap), compact link messages or dense links (fractal heap and v2
  B-tree name index, which ``libver='latest'`` uses past eight links); contiguous and compact dataset
  layouts; fixed-point, floating-point, fixed and variable-length strings (global heap), enums
  (h5py's booleans) and opaque types (mosaic's ``bytes``); attribute messages v1-v3. Dense
  attribute storage, multi-level heaps or name indexes and chunked layouts raise
  NotImplementedError;
* writing: superblock v0 with v1 object headers, symbol-table groups, contiguous datasets and
  attributes, strings as fixed-length UTF-8, booleans as h5py's FALSE/TRUE enum.

``HDF5``, ``file_exists``, ``write``/``read`` and the description layout (groups with an
``is_array`` attribute, ``<name>_%08d`` members for lists of dicts, datasets tagged
``is_ndarray/is_list/is_tuple/is_str/is_bytes/is_none``) follow mosaic's module (h5.py:39-398).
Checksums of v2 structures are not verified.
"""

import datetime
import mmap
import os
import tempfile
import re
import struct

import numpy as np

__all__ = ['HDF5', 'File', 'Dataset', 'Struct', 'file_exists', 'write_file', 'read_file']

_SIGNATURE = b'\x89HDF\r\n\x1a\n'
_UNDEF = 0xFFFFFFFFFFFFFFFF
_PROTOCOL_VERSION = '0.1'


class Struct(dict):
    """Dict with attribute access, as mosaic.types.Struct (struct.py:9-70) presents a loaded
    description; nested dicts are Structs too."""

    def __init__(self, content=None):
        super().__init__()
        for k, v in (content or {}).items():
            if isinstance(v, dict) and not isinstance(v, Struct):
                v = Struct(v)
            elif isinstance(v, list) and v and all(isinstance(o, dict) for o in v):
                v = [o if isinstance(o, Struct) else Struct(o) for o in v]
            self[k] = v

    def __getattr__(self, item):
        try:
            return self[item]
        except KeyError:
            raise AttributeError(item) from None

    def __setattr__(self, key, value):
        self[key] = value


# ------------------------------------------------------------------------------------- reading

class Dataset:
    """A dataset of an opened file: ``attrs``, ``shape``, ``dtype``; ``ds[()]`` or ``load()`` reads
    it (the lazy form mosaic hands out for ndarrays, h5.py:182-190)."""

    def __init__(self, name, attrs, shape, dtype, reader):
        self.name = name
        self.attrs = attrs
        self.shape = shape
        self.dtype = dtype
        self._reader = reader

    def __getitem__(self, key):
        if key != () and key != Ellipsis:
            return self._reader()[key]
        return self._reader()

    def load(self):
        return self._reader()


class Group(dict):
    """A group of an opened file: its members by name and its ``attrs``."""

    def __init__(self, name, attrs):
        super().__init__()
        self.name = name
        self.attrs = attrs


class _Type:
    """A decoded datatype message: kind in {'num', 'str', 'vstr', 'enum', 'opaque'}."""

    def __init__(self, kind, size, dtype=None, members=None, charset=0):
        self.kind, self.size, self.dtype, self.members, self.charset = kind, size, dtype, members, charset


class _Closed:
    """The bytes of a closed File: any read raises a ValueError naming the file."""

    def __init__(self, filename):
        self.filename = filename

    def __getitem__(self, key):
        raise ValueError('HDF5 file %s is closed: load its datasets before closing it' % self.filename)

    def __len__(self):
        return 0


class File:
    """Read-only view of an HDF5 file, memory-mapped (datasets are read when loaded); ``root`` is
    the root Group."""

    def __init__(self, filename):
        with open(filename, 'rb') as fh:
            size = os.fstat(fh.fileno()).st_size
            self._b = mmap.mmap(fh.fileno(), 0, access=mmap.ACCESS_READ) if size else b''
        self.filename = filename
        self._gheaps = {}
        self._path = set()  # object headers on the path from the root (hard links may form cycles)
        self._superblock()
        self.root = self._object('/', self._root_addr, None)

    def __getitem__(self, path):
        node = self.root
        for part in [p for p in path.split('/') if p]:
            node = node[part]
        return node

    def close(self):
        """Unmaps the file; datasets not yet loaded can no longer be read (ValueError)."""
        if isinstance(self._b, mmap.mmap):
            self._b.close()
        self._b = _Closed(self.filename)

    # ---- primitives
    def _u(self, pos, n):
        return int.from_bytes(self._b[pos:pos + n], 'little')

    def _addr(self, pos):
        return self._u(pos, self.O)

    def _abs(self, a):
        return a + self._base

    def _need(self, pos, sig):
        if self._b[pos:pos + 4] != sig:
            raise ValueError('HDF5: expected %r at %d' % (sig, pos))

    def _cstr(self, pos):
        end = self._b.find(b'\0', pos)
        if end < 0:
            raise ValueError('HDF5: unterminated string at %d' % pos)
        return self._b[pos:end]

    # ---- superblock
    def _superblock(self):
        pos = 0
        while self._b[pos:pos + 8] != _SIGNATURE:
            pos = 512 if pos == 0 else 2 * pos
            if pos + 8 > len(self._b):
                raise ValueError('not an HDF5 file')
        ver = self._b[pos + 8]
        if ver in (0, 1):
            self.O, self.L = self._b[pos + 13], self._b[pos + 14]
            q = pos + 24 + (4 if ver == 1 else 0)
            self._base = self._addr(q)
            entry = q + 4 * self.O  # base, free-space, end-of-file, driver
            self._root_addr = self._abs(self._addr(entry + self.O))
        elif ver in (2, 3):
            self.O, self.L = self._b[pos + 9], self._b[pos + 10]
            q = pos + 12
            self._base = self._addr(q)
            self._root_addr = self._abs(self._addr(q + 3 * self.O))
        else:
            raise NotImplementedError('HDF5 superblock version %d' % ver)

    # ---- object headers
    def _messages(self, addr):
        """(type, data position, size) of every message of the object header at addr."""
        out = []
        if self._b[addr:addr + 4] == b'OHDR':
            flags = self._b[addr + 5]
            q = addr + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
            nsz = 1 << (flags & 3)
            size0 = self._u(q, nsz)
            q += nsz
            blocks = [(q, q + size0)]
            seen = set()
            hdr = 6 if flags & 0x04 else 4
            while blocks:
                q, end = blocks.pop(0)
                while q + hdr <= end:
                    mtype, msize = self._b[q], self._u(q + 1, 2)
                    d = q + hdr
                    if mtype == 0x10:
                        c = self._abs(self._addr(d))
                        self._need(c, b'OCHK')
                        if c in seen:
                            raise ValueError('HDF5: object header continuation loop at %d' % c)
                        seen.add(c)
                        blocks.append((c + 4, c + self._u(d + self.O, self.L) - 4))
                    elif mtype != 0:
                        out.append((mtype, d, msize))
                    q = d + msize
            return out
        if self._b[addr] != 1:
            raise NotImplementedError('HDF5 object header version %d' % self._b[addr])
        nmsg = self._u(addr + 2, 2)
        blocks = [(addr + 16, addr + 16 + self._u(addr + 8, 4))]
        seen = set()
        while blocks and len(out) < nmsg:
            q, end = blocks.pop(0)
            while q + 8 <= end:
                mtype, msize = self._u(q, 2), self._u(q + 2, 2)
                d = q + 8
                if mtype == 0x10:
                    c = self._abs(self._addr(d))
                    if c in seen:
                        raise ValueError('HDF5: object header continuation loop at %d' % c)
                    seen.add(c)
                    blocks.append((c, c + self._u(d + self.O, self.L)))
                elif mtype != 0:
                    out.append((mtype, d, msize))
                q = d + msize
        return out

    def _object(self, name, addr, parent):
        if addr in self._path:
            raise ValueError('HDF5: hard link cycle at %r' % name)
        self._path.add(addr)
        try:
            return self._object_at(name, addr)
        finally:
            self._path.discard(addr)

    def _object_at(self, name, addr):
        msgs = self._messages(addr)
        attrs = {}
        for t, d, _ in msgs:
            if t == 0x0C:
                k, v = self._attribute(d)
                attrs[k] = v
            elif t == 0x15 and self._u(d + 2 + (2 if self._b[d + 1] & 1 else 0), self.O) != _UNDEF:
                raise NotImplementedError('HDF5 dense attribute storage')
        types = {t for t, _, _ in msgs}
        if 0x11 in types or 0x06 in types or 0x02 in types:
            g = Group(name, attrs)
            for t, d, _ in msgs:
                if t == 0x11:
                    self._symbol_table(g, self._abs(self._addr(d)), self._abs(self._addr(d + self.O)))
                elif t == 0x06:
                    lname, target = self._link(d)
                    if target is not None:
                        g[lname] = self._object(lname, target, g)
                elif t == 0x02:
                    q = d + 2 + (8 if self._b[d + 1] & 1 else 0)
                    heap, index = self._addr(q), self._addr(q + self.O)
                    if heap != _UNDEF:  # dense storage: link messages in a fractal heap, by name index
                        for lname, target in self._dense_links(self._abs(heap), self._abs(index)):
                            if target is not None:
                                g[lname] = self._object(lname, target, g)
            return g
        if 0x08 in types:
            return self._dataset(name, msgs, attrs)
        return Group(name, attrs)  # an object with neither links nor layout (empty group)

    def _symbol_table(self, g, btree, heap):
        self._need(heap, b'HEAP')
        data = self._abs(self._addr(heap + 8 + 2 * self.L))

        def walk(node, above=256):
            self._need(node, b'TREE')
            level, used = self._b[node + 5], self._u(node + 6, 2)
            if level >= above:
                raise ValueError('HDF5: group B-tree levels do not decrease at %d' % node)
            q = node + 8 + 2 * self.O
            for i in range(used):
                child = self._abs(self._addr(q + self.L + i * (self.L + self.O)))
                if level > 0:
                    walk(child, level)
                    continue
                self._need(child, b'SNOD')
                for k in range(self._u(child + 6, 2)):
                    e = child + 8 + k * (2 * self.O + 24)
                    lname = self._cstr(data + self._addr(e)).decode('utf-8')
                    g[lname] = self._object(lname, self._abs(self._addr(e + self.O)), g)

        walk(btree)

    def _dense_links(self, heap, index):
        """Links of a group with dense storage: the records of its v2 B-tree name index (type 5:
        name hash, heap ID) point at link messages stored as managed objects of its fractal heap.
        Handles a root direct block or a root indirect block of direct blocks, and a name index
        whose root is a leaf (the shape of every group short of thousands of links)."""
        self._need(heap, b'FRHP')
        flags = self._b[heap + 9]
        max_managed = self._u(heap + 10, 4)
        L, O = self.L, self.O
        if self._u(heap + 7, 2):
            raise NotImplementedError('HDF5 fractal heap with I/O filters')
        q = heap + 14 + 10 * L + 2 * O  # table width, past the object counters
        width = self._u(q, 2)
        start_block, max_direct = self._u(q + 2, L), self._u(q + 2 + L, L)
        max_heap_bits = self._u(q + 2 + 2 * L, 2)
        root = self._addr(q + 2 + 2 * L + 4)
        rows = self._u(q + 2 + 2 * L + 4 + O, 2)
        off_bytes = (max_heap_bits + 7) // 8
        len_bytes = min((max_direct.bit_length() - 1 + 7) // 8, (max_managed.bit_length() - 1) // 8 + 1)
        hdr = 5 + O + off_bytes + (4 if flags & 2 else 0)  # direct block header

        blocks = []  # (heap offset, address, size) of every direct block
        if rows == 0:
            blocks.append((0, self._abs(root), start_block))
        else:
            r = self._abs(root)
            self._need(r, b'FHIB')
            direct_rows = (max_direct.bit_length() - 1) - (start_block.bit_length() - 1) + 2
            if rows > direct_rows:
                raise NotImplementedError('HDF5 fractal heap with indirect child blocks')
            e, off = r + 5 + O + off_bytes, 0
            for row in range(rows):
                size = start_block if row < 2 else start_block << (row - 1)
                for _ in range(width):
                    a = self._addr(e)
                    e += O
                    if a != _UNDEF:
                        blocks.append((off, self._abs(a), size))
                    off += size

        def managed(hid):
            if (hid[0] >> 4) & 3 != 0:
                raise NotImplementedError('HDF5 huge or tiny fractal heap objects')
            off = int.from_bytes(hid[1:1 + off_bytes], 'little')
            n = int.from_bytes(hid[1 + off_bytes:1 + off_bytes + len_bytes], 'little')
            for boff, a, size in blocks:
                if boff <= off < boff + size:
                    self._need(a, b'FHDB')
                    if off - boff < hdr or off + n > boff + size:
                        break
                    return a + (off - boff)
            raise ValueError('HDF5: fractal heap offset %d outside its blocks' % off)

        self._need(index, b'BTHD')
        rec_size, depth = self._u(index + 10, 2), self._u(index + 12, 2)
        node, nrec = self._abs(self._addr(index + 16)), self._u(index + 16 + O, 2)
        if depth != 0:
            raise NotImplementedError('HDF5 link name index deeper than one leaf')
        if nrec == 0:
            return []
        self._need(node, b'BTLF')
        out = []
        for i in range(nrec):
            rec = node + 6 + i * rec_size
            out.append(self._link(managed(self._b[rec + 4:rec + rec_size])))
        return out

    def _link(self, d):
        flags = self._b[d + 1]
        q = d + 2
        ltype = 0
        if flags & 0x08:
            ltype = self._b[q]
            q += 1
        if flags & 0x04:
            q += 8
        if flags & 0x10:
            q += 1
        nsz = 1 << (flags & 3)
        n = self._u(q, nsz)
        q += nsz
        lname = self._b[q:q + n].decode('utf-8')
        q += n
        if ltype != 0:
            return lname, None  # soft and external links are not followed
        return lname, self._abs(self._addr(q))

    # ---- datatypes, dataspaces, data
    def _datatype(self, d):
        """(_Type, size of the message)."""
        cls, ver = self._b[d] & 0x0F, self._b[d] >> 4
        bits = self._u(d + 1, 3)
        size = self._u(d + 4, 4)
        p = d + 8
        order = '>' if bits & 1 else '<'
        if cls == 0:
            dt = np.dtype('%s%s%d' % (order, 'i' if bits & 0x08 else 'u', size))
            return _Type('num', size, dt), 12
        if cls == 1:
            if size not in (2, 4, 8):
                raise NotImplementedError('HDF5 %d-byte float' % size)
            return _Type('num', size, np.dtype('%sf%d' % (order, size))), 20
        if cls == 3:
            return _Type('str', size, np.dtype('S%d' % size), charset=(bits >> 4) & 0xF), 8
        if cls == 5:
            return _Type('opaque', size, np.dtype('V%d' % size)), 8 + (bits & 0xFF)
        if cls == 8:
            base, bsize = self._datatype(p)
            q = p + bsize
            n = bits & 0xFFFF
            names = []
            for _ in range(n):
                s = self._cstr(q)
                names.append(s.decode('utf-8'))
                q += len(s) + 1 if ver >= 3 else (len(s) + 8) // 8 * 8
            vals = np.frombuffer(self._b[q:q + n * base.size], base.dtype)
            return _Type('enum', size, base.dtype, dict(zip(names, vals.tolist()))), q + n * base.size - d
        if cls == 9:
            if bits & 0xF != 1:
                raise NotImplementedError('HDF5 variable-length sequences')
            _, bsize = self._datatype(p)
            return _Type('vstr', size, charset=(bits >> 8) & 0xF), 8 + bsize
        raise NotImplementedError('HDF5 datatype class %d' % cls)

    def _dataspace(self, d):
        ver, rank = self._b[d], self._b[d + 1]
        if ver == 1:
            q = d + 8
        else:
            q = d + 4
            if self._b[d + 3] == 2:
                return None  # null dataspace
        return tuple(self._u(q + i * self.L, self.L) for i in range(rank))

    def _gheap(self, addr, index):
        if addr not in self._gheaps:
            self._need(addr, b'GCOL')
            objs, q = {}, addr + 16
            end = addr + self._u(addr + 8, self.L)
            while q + 8 + self.L <= end:
                idx, size = self._u(q, 2), self._u(q + 8, self.L)
                if idx == 0:
                    break
                objs[idx] = self._b[q + 8 + self.L:q + 8 + self.L + size]
                q += 8 + self.L + (size + 7) // 8 * 8
            self._gheaps[addr] = objs
        return self._gheaps[addr][index]

    def _values(self, t, shape, raw, as_str):
        n = int(np.prod(shape)) if shape else 1
        if t.kind == 'vstr':
            out = []
            for i in range(n):
                e = raw[i * t.size:(i + 1) * t.size]
                length = int.from_bytes(e[0:4], 'little')
                a = int.from_bytes(e[4:4 + self.O], 'little')
                idx = int.from_bytes(e[4 + self.O:8 + self.O], 'little')
                s = b'' if length == 0 else self._gheap(self._abs(a), idx)[:length]
                out.append(s.decode('utf-8') if as_str else s)
            arr = np.empty(n, dtype=object)
            arr[:] = out
            return arr[0] if shape == () else arr.reshape(shape)
        if t.kind == 'enum':
            vals = np.frombuffer(raw[:n * t.size], t.dtype)
            if sorted(t.members.items()) == [('FALSE', 0), ('TRUE', 1)]:
                vals = vals.astype(np.bool_)
        else:
            vals = np.frombuffer(raw[:n * t.size], t.dtype)
        if t.kind == 'str' and t.charset == 1 and as_str:
            vals = np.array([v.decode('utf-8') for v in vals], dtype=object)
        if shape == ():
            return vals[0]
        return vals.reshape(shape).copy()

    def _attribute(self, d):
        ver = self._b[d]
        nsz, tsz, ssz = self._u(d + 2, 2), self._u(d + 4, 2), self._u(d + 6, 2)
        q = d + 8 + (1 if ver == 3 else 0)
        pad = (lambda x: (x + 7) // 8 * 8) if ver == 1 else (lambda x: x)
        name = self._b[q:q + nsz].rstrip(b'\0').decode('utf-8')
        q += pad(nsz)
        t, _ = self._datatype(q)
        q += pad(tsz)
        shape = self._dataspace(q)
        q += pad(ssz)
        if shape is None:
            return name, None
        n = int(np.prod(shape)) if shape else 1
        return name, self._values(t, shape, self._b[q:q + n * t.size], as_str=True)

    def _dataset(self, name, msgs, attrs):
        t = shape = layout = None
        for mt, d, _ in msgs:
            if mt == 0x03:
                t, _ = self._datatype(d)
            elif mt == 0x01:
                shape = self._dataspace(d)
            elif mt == 0x08:
                layout = d
            elif mt == 0x0B:
                raise NotImplementedError('HDF5 filters (compressed datasets)')
        ver, cls = self._b[layout], self._b[layout + 1]
        if ver < 3:
            raise NotImplementedError('HDF5 data layout version %d' % ver)
        n = int(np.prod(shape)) if shape else (0 if shape is None else 1)
        nbytes = n * t.size
        if cls == 0:
            start = layout + 4
        elif cls == 1:
            a = self._addr(layout + 2)
            start = None if a == _UNDEF else self._abs(a)
        else:
            raise NotImplementedError('HDF5 chunked or virtual datasets')

        def read():  # the data are sliced out of the mapping only when the dataset is loaded
            if shape is None:
                return None
            raw = b'\0' * nbytes if start is None else self._b[start:start + nbytes]
            return self._values(t, shape, raw, as_str=False)

        dt = np.dtype(object) if t.kind == 'vstr' else (np.dtype(np.bool_) if t.kind == 'enum' else t.dtype)
        return Dataset(name, attrs, shape if shape is not None else (), dt, read)


def read_file(filename):
    """The root Group of an HDF5 file (its datasets read when loaded, from the file's mapping)."""
    return File(filename).root


# ------------------------------------------------------------------------------------- writing

def _pad8(b):
    return b + b'\0' * ((-len(b)) % 8)


def _dtype_message(kind, arg):
    """Datatype message bytes: kind 'num' (a numpy dtype), 'bool', 'str' (length) or 'opaque'."""
    if kind == 'bool':
        base = _dtype_message('num', np.dtype(np.int8))
        names = _pad8(b'FALSE\0') + _pad8(b'TRUE\0')
        return struct.pack('<B3sI', 0x18, (2).to_bytes(3, 'little'), 1) + base + names + b'\x00\x01'
    if kind == 'str':
        return struct.pack('<B3sI', 0x13, bytes([0x11, 0, 0]), max(1, arg))  # null-padded, UTF-8
    if kind == 'opaque':
        tag = _pad8(b'bytes\0')
        return struct.pack('<B3sI', 0x15, bytes([len(tag), 0, 0]), arg) + tag
    dt = np.dtype(arg).newbyteorder('<')
    if dt.kind in 'iu':
        bits = bytes([0x08 if dt.kind == 'i' else 0, 0, 0])
        return struct.pack('<B3sIHH', 0x10, bits, dt.itemsize, 0, 8 * dt.itemsize)
    if dt.kind == 'f':
        e_loc, e_size, m_size, bias = {2: (10, 5, 10, 15), 4: (23, 8, 23, 127), 8: (52, 11, 52, 1023)}[dt.itemsize]
        bits = bytes([0x20, 8 * dt.itemsize - 1, 0])
        return struct.pack('<B3sIHHBBBBI', 0x11, bits, dt.itemsize, 0, 8 * dt.itemsize, e_loc, e_size, 0, m_size,
                           bias)
    raise TypeError('cannot store dtype %s in HDF5' % dt)


def _encode(value):
    """(datatype message, shape, raw bytes) of a value as mosaic stores it."""
    if isinstance(value, (bytes, np.void)):
        b = bytes(value)
        return _dtype_message('opaque', max(1, len(b))), (), b if b else b'\0'
    arr = np.asarray(value)
    if arr.dtype.kind in 'US' or arr.dtype == object:
        items = [v if isinstance(v, bytes) else str(v).encode('utf-8') for v in arr.reshape(-1).tolist()]
        size = max([1] + [len(v) for v in items])
        raw = b''.join(v.ljust(size, b'\0') for v in items)
        return _dtype_message('str', size), arr.shape, raw
    if arr.dtype.kind == 'b':
        return _dtype_message('bool', None), arr.shape, arr.astype(np.int8).tobytes()
    if arr.dtype.kind == 'c':
        raise TypeError('complex data is not supported by this HDF5 writer')
    arr = np.ascontiguousarray(arr, dtype=arr.dtype.newbyteorder('<'))
    return _dtype_message('num', arr.dtype), arr.shape, arr.tobytes()


def _dataspace_message(shape):
    return struct.pack('<BBBBI', 1, len(shape), 0, 0, 0) + b''.join(struct.pack('<Q', d) for d in shape)


def _attribute_message(name, value):
    tmsg, shape, raw = _encode(value)
    smsg = _dataspace_message(shape)
    nm = name.encode('utf-8') + b'\0'
    return struct.pack('<BBHHH', 1, 0, len(nm), len(tmsg), len(smsg)) + _pad8(nm) + _pad8(tmsg) + _pad8(smsg) + raw


class _Writer:
    """Lays out a file in memory: superblock v0, then objects at 8-byte aligned addresses."""

    GROUP_INTERNAL_K = 16

    def __init__(self, leaf_k):
        self.leaf_k = leaf_k
        self.buf = bytearray(96)  # superblock v0 with the root symbol table entry

    def alloc(self, data):
        self.buf += b'\0' * ((-len(self.buf)) % 8)
        a = len(self.buf)
        self.buf += data
        return a

    def header(self, messages):
        """Object header v1 holding (type, data) messages."""
        body = b''
        for t, data in messages:
            data = _pad8(data)
            body += struct.pack('<HHB3s', t, len(data), 0, b'\0\0\0') + data
        return self.alloc(struct.pack('<BBHII4s', 1, 0, len(messages), 1, len(body), b'\0' * 4) + body)

    def dataset(self, value, attrs):
        tmsg, shape, raw = _encode(value)
        addr = self.alloc(raw) if raw else _UNDEF
        msgs = [(0x01, _dataspace_message(shape)), (0x03, tmsg),
                (0x05, bytes([2, 2, 2, 1, 0, 0, 0, 0])),  # fill value v2: late allocation, default (size 0)
                (0x08, struct.pack('<BBQQ', 3, 1, addr, len(raw)))]
        msgs += [(0x0C, _attribute_message(k, v)) for k, v in attrs.items()]
        return self.header(msgs)

    def group(self, members, attrs):
        """members: [(name, object header address, (B-tree, heap) of a subgroup or None)];
        returns (header address, B-tree, heap)."""
        members = sorted(members, key=lambda m: m[0].encode('utf-8'))
        names = b'\0' * 8
        offsets = []
        for n, _, _ in members:
            offsets.append(len(names))
            names += _pad8(n.encode('utf-8') + b'\0')
        data = self.alloc(names)
        # free-list head 1: libhdf5's on-disk end-of-list marker (no free block)
        heap = self.alloc(b'HEAP' + struct.pack('<B3sQQQ', 0, b'\0' * 3, len(names), 1, data))
        cap = 2 * self.leaf_k
        snod = b'SNOD' + struct.pack('<BBH', 1, 0, len(members))
        for (_, oh, stab), off in zip(members, offsets):  # subgroups cache their B-tree and heap (type 1)
            scratch = struct.pack('<QQ', *stab) if stab else b'\0' * 16
            snod += struct.pack('<QQII16s', off, oh, 1 if stab else 0, 0, scratch)
        snod += b'\0' * ((cap - len(members)) * 40)
        ik = self.GROUP_INTERNAL_K
        tree = b'TREE' + struct.pack('<BBHQQ', 0, 0, 1 if members else 0, _UNDEF, _UNDEF)
        if members:
            tree += struct.pack('<QQQ', 0, self.alloc(snod), offsets[-1])
        tree += b'\0' * (24 + (2 * ik + 1) * 8 + 2 * ik * 8 - len(tree))
        btree = self.alloc(tree)
        msgs = [(0x11, struct.pack('<QQ', btree, heap))]
        msgs += [(0x0C, _attribute_message(k, v)) for k, v in attrs.items()]
        return self.header(msgs), btree, heap

    def finish(self, root, btree, heap):
        sb = _SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack('<HHI', self.leaf_k, self.GROUP_INTERNAL_K, 0)
        sb += struct.pack('<QQQQ', 0, _UNDEF, len(self.buf), _UNDEF)
        sb += struct.pack('<QQII', 0, root, 1, 0) + struct.pack('<QQ', btree, heap)
        self.buf[0:96] = sb
        return bytes(self.buf)


def _build(name, obj):
    """(attrs, members) for a group or ('dataset', value, attrs), after mosaic's write (h5.py:39-119)."""
    if isinstance(obj, dict):
        attrs = {}
        if name == '/':
            attrs['protocol'] = _PROTOCOL_VERSION
            attrs['datetime'] = str(datetime.datetime.now())
        attrs['is_array'] = False
        return attrs, [(k, _build(k, v)) for k, v in obj.items()]
    if isinstance(obj, list) and len(obj) > 0 and isinstance(obj[0], dict):
        return {'is_array': True, 'len': len(obj)}, [('%s_%08d' % (name, i), _build('%s_%08d' % (name, i), o))
                                                      for i, o in enumerate(obj)]
    is_bytes = isinstance(obj, bytes)
    is_none = obj is None
    value = 'None' if is_none else obj
    attrs = {'is_ndarray': isinstance(value, np.ndarray), 'is_list': isinstance(value, list),
             'is_tuple': isinstance(value, tuple), 'is_str': isinstance(value, str), 'is_bytes': is_bytes,
             'is_none': is_none}
    if not isinstance(value, np.ndarray) and not is_bytes:
        flat = np.asarray(value).flatten().tolist()
        attrs['is_str'] = bool(flat) and isinstance(flat[0], str)
    return ('dataset', value, attrs)


def write_file(filename, description):
    """Write a mosaic description (nested dicts) as an HDF5 file."""
    tree = _build('/', description)

    def count(node):
        if isinstance(node, tuple) and len(node) == 2:
            return max([len(node[1])] + [count(v) for _, v in node[1]])
        return 0

    w = _Writer(max(4, (count(tree) + 1) // 2))

    def emit(node):
        """(object header address, (B-tree, heap) for a group or None)."""
        if len(node) == 3:
            return w.dataset(node[1], node[2]), None
        attrs, members = node
        oh, btree, heap = w.group([(k,) + emit(v) for k, v in members], attrs)
        return oh, (btree, heap)

    oh, (btree, heap) = emit(tree)
    data = w.finish(oh, btree, heap)
    # written beside the target and renamed over it: a File still mapping the old file keeps its
    # inode, so its lazy datasets stay readable (truncating in place would fault their pages)
    folder = os.path.dirname(os.path.abspath(filename))
    fd, tmp = tempfile.mkstemp(prefix='.' + os.path.basename(filename) + '.', suffix='.tmp', dir=folder)
    try:
        with os.fdopen(fd, 'wb') as fh:
            fh.write(data)
        umask = os.umask(0)
        os.umask(umask)
        os.chmod(tmp, 0o666 & ~umask)  # the permissions open(filename, 'wb') would give
        os.replace(tmp, filename)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise


# ------------------------------------------------------------------------------------- mosaic's layer

def _decode_list(items):
    return [_decode_list(v) if isinstance(v, list) else (v.decode('utf-8') if isinstance(v, bytes) else v)
            for v in items]


class FilterException(Exception):
    pass


def _read(obj, lazy=True, filter=None, only=None):
    """mosaic's read (h5.py:127-174) over this module's Group/Dataset."""
    if isinstance(obj, Group):
        filter = {} if filter is None else filter

        def member(key):
            if filter and key in filter:
                return _read(obj[key], lazy=lazy, filter=filter, only=filter[key])
            return _read(obj[key], lazy=lazy, filter=filter)

        keys = sorted(obj.keys()) if obj.attrs.get('is_array') else list(obj.keys())
        out = [] if obj.attrs.get('is_array') else {}
        for key in keys:
            if only is not None and key not in only:
                continue
            try:
                value = member(key)
            except FilterException:
                continue
            if isinstance(out, list):
                out.append(value)
            else:
                out[key] = value
        return out
    return _read_dataset(obj, lazy=lazy)


def _read_dataset(obj, lazy=True):
    """mosaic's _read_dataset (h5.py:177-216)."""
    a = obj.attrs
    if a.get('is_none'):
        return None
    if a.get('is_ndarray'):
        return obj if lazy else obj[()]
    if a.get('is_bytes'):
        return obj[()].tobytes()
    data = obj[()]
    if a.get('is_str') and not a.get('is_list'):
        return data.decode('utf-8') if isinstance(data, bytes) else str(data)
    if a.get('is_tuple'):
        return tuple(data)
    if a.get('is_list'):
        data = list(data.tolist())
        return _decode_list(data) if a.get('is_str') else data
    return data.item() if hasattr(data, 'item') else data


def _merge(old, new):
    for k, v in new.items():
        if isinstance(v, dict) and isinstance(old.get(k), dict):
            _merge(old[k], v)
        elif isinstance(v, list) and v and isinstance(v[0], dict) and isinstance(old.get(k), list):
            old[k] = list(old[k]) + list(v)
        else:
            old[k] = v
    return old


def _camel_case(name):
    """mosaic.utils.change_case.camel_case (change_case.py:29-47)."""
    name = re.sub(r'^[_.]', '', str(name))
    if not name:
        return name
    return name[0].upper() + re.sub(r'[_.\s]([a-zA-Z0-9])', lambda m: m.group(1).upper(), name[1:])


def _filename(args, kwargs, reading):
    filename = args[0] if args else kwargs.pop('filename', None)
    path = kwargs.pop('path', None) or os.getcwd()
    if filename is not None:
        return filename if os.path.isabs(filename) else os.path.join(path, filename)
    project, parameter = kwargs.pop('project_name', None), kwargs.pop('parameter', None)
    if project is None or parameter is None:
        raise RuntimeError('Either filename or project_name and parameter are needed to generate a filename')
    param = _camel_case(parameter)
    ext = kwargs.pop('extension', '.h5')
    version = kwargs.pop('version', None)

    def name(v):
        return os.path.join(path, '%s-%s-%05d%s' % (project, param, v, ext) if v > 0 else '%s-%s%s' % (project,
                                                                                                      param, ext))

    if version is None or version < 0:
        version = kwargs.pop('version_start', 0)
        while os.path.exists(name(version)):
            version += 1
        if reading:
            version -= 1
    return name(version)


class HDF5:
    """mosaic.file_manipulation.h5.HDF5 (h5.py:219-338): open by ``filename`` (and ``path``) or by
    ``project_name``/``parameter``/``version``/``extension`` with mosaic's naming
    (``<project>-<Parameter>[-%05d]<ext>``, the latest version when none is given); ``mode`` 'r',
    'w' or 'a'. ``load`` returns the description as a Struct, ``dump`` writes it, ``append``
    merges it into the file's."""

    def __init__(self, *args, **kwargs):
        self._mode = kwargs.pop('mode')
        self._filename = _filename(args, kwargs, self._mode.startswith('r'))
        self._file = File(self._filename) if self._mode.startswith('r') else None

    @property
    def mode(self):
        return self._mode

    @property
    def filename(self):
        return self._filename

    @property
    def file(self):
        return self._file

    def close(self):
        """Closes the file: lazily returned datasets not yet loaded become unreadable, as with h5py."""
        if self._file is not None:
            self._file.close()
        self._file = None

    def load(self, lazy=True, filter=None, only=None):
        if filter is not None:
            filter = {k: [v_ if isinstance(v_, str) else str(v_) for v_ in (v if isinstance(v, list) else [v])]
                      for k, v in filter.items()}
        if self._file is not None:
            return Struct(_read(self._file.root, lazy=lazy, filter=filter, only=only))
        f = File(self._filename)  # mode 'w' / 'a': a view of the file as it is now
        if lazy:
            return Struct(_read(f.root, lazy=True, filter=filter, only=only))
        try:  # everything read into memory: the mapping is not needed afterwards
            return Struct(_read(f.root, lazy=False, filter=filter, only=only))
        finally:
            f.close()

    def dump(self, description):
        write_file(self._filename, description)

    def append(self, description):
        old = {}
        if os.path.exists(self._filename):
            f = File(self._filename)
            try:  # everything read into memory, and the mapping closed, before the file is rewritten
                old = _read(f.root, lazy=False)
            finally:
                f.close()
        write_file(self._filename, _merge(old, description))

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc_val, exc_tb):
        self.close()


def file_exists(*args, **kwargs):
    """mosaic.file_manipulation.h5.file_exists (h5.py:341-398)."""
    kwargs = dict(kwargs)
    if not args and kwargs.get('filename') is None and kwargs.get('version') is None:
        kwargs['version'] = 0
    return os.path.exists(_filename(args, kwargs, False))
