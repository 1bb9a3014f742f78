"""The HDF5 layer (stride_gb300/h5.py) that stands in for mosaic's h5py-based one
(mosaic/file_manipulation/h5.py): the reference's own libhdf5-written model file decoded against
its golden summary, writer output checked field by field against the encodings libhdf5 used in
that file, round trips of every value kind mosaic stores, mosaic's file naming, a hand-built
superblock-v3 file for the v2 object-header paths, and the problem model's dump/load."""

import json
import os
import struct

import numpy as np
import pytest

from stride_gb300 import fwi, h5, problem

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, 'golden', 'anastasio2d_truemodel.json')


def _fixture():
    from tests.golden import make_h5_golden
    return make_h5_golden.FIXTURE


@pytest.mark.skipif(not os.path.exists(_fixture()), reason='the reference checkout is not present')
def test_reference_model_file_matches_golden():
    from tests.golden import make_h5_golden
    with open(GOLDEN) as fh:
        golden = json.load(fh)
    assert make_h5_golden.summary(_fixture()) == golden


def test_golden_summary_is_the_breast2d_grid():
    with open(GOLDEN) as fh:
        g = json.load(fh)
    assert g['shape'] == [356, 385] and g['extended_shape'] == [456, 485]
    assert g['space']['extra'] == [50, 50] and g['space']['absorbing'] == [40, 40]
    assert 1400 <= g['data']['min'] <= g['data']['max'] <= 1700


def _description():
    rng = np.random.default_rng(3)
    return {
        'space': {'shape': (40, 52), 'spacing': (0.5e-3, 0.5e-3), 'extra': (8, 8), 'absorbing': (6, 6)},
        'time': {'start': 0.0, 'stop': 1e-4, 'step': 8e-8, 'num': 1251},
        'data': rng.standard_normal((40, 52)).astype(np.float32),
        'data64': rng.standard_normal(7),
        'ints16': np.arange(-3, 3, dtype=np.int16), 'uints': np.arange(4, dtype=np.uint32),
        'mask': np.array([True, False, True]),
        'inner': [['8', '48', 'None'], ['8', '60', 'None']],
        'dtype': 'float32', 'name': 'vp é', 'count': 12, 'ratio': 0.25, 'flag': True,
        'shape': (40, 52), 'ids': [3, 1, 2], 'blob': b'\x00\x01raw', 'nothing': None,
        'empty': np.zeros((0, 4), np.float32),
        'shots': [{'id': k, 'coords': rng.standard_normal((2, 2))} for k in range(3)],
    }


def test_round_trip_of_every_value_kind(tmp_path):
    desc = _description()
    path = str(tmp_path / 'd.h5')
    h5.write_file(path, desc)
    got = h5.HDF5(path, mode='r').load(lazy=False)
    assert sorted(got.keys()) == sorted(desc.keys())
    for k in ('data', 'data64', 'ints16', 'uints', 'mask', 'empty'):
        assert got[k].dtype == desc[k].dtype and np.array_equal(got[k], desc[k])
    assert got.inner == desc['inner'] and got.dtype == 'float32' and got.name == desc['name']
    assert got.count == 12 and got.ratio == 0.25 and got.flag is True
    assert got.shape == (40, 52) and isinstance(got.shape, tuple) and got.ids == [3, 1, 2]
    assert got.blob == desc['blob'] and got.nothing is None
    assert got.space.spacing == (0.5e-3, 0.5e-3) and got.time.num == 1251
    assert [s.id for s in got.shots] == [0, 1, 2]
    for a, b in zip(got.shots, desc['shots']):
        assert np.array_equal(a.coords, b['coords'])
    lazy = h5.HDF5(path, mode='r').load()
    assert isinstance(lazy.data, h5.Dataset) and np.array_equal(lazy.data.load(), desc['data'])


def test_many_members_and_deep_groups(tmp_path):
    desc = {'m%03d' % k: {'v': np.full(3, k, np.int64)} for k in range(40)}
    desc['deep'] = {'a': {'b': {'c': {'d': 'leaf'}}}}
    path = str(tmp_path / 'm.h5')
    h5.write_file(path, desc)
    got = h5.HDF5(path, mode='r').load(lazy=False)
    assert all(np.array_equal(got['m%03d' % k].v, np.full(3, k)) for k in range(40))
    assert got.deep.a.b.c.d == 'leaf'
    with open(path, 'rb') as fh:
        b = fh.read()
    assert struct.unpack('<H', b[16:18])[0] >= 21  # group leaf K sized for 41 members in one node


def test_writer_structures_match_libhdf5_encodings(tmp_path):
    """Superblock v0, root entry, local heap, B-tree and symbol-table nodes, and the float and
    boolean datatype messages, as libhdf5 wrote them in the reference's model file."""
    path = str(tmp_path / 's.h5')
    h5.write_file(path, {'x': np.ones(2, np.float32), 'g': {'flag': False}})
    with open(path, 'rb') as fh:
        b = fh.read()
    assert b[:8] == b'\x89HDF\r\n\x1a\n'
    assert list(b[8:16]) == [0, 0, 0, 0, 0, 8, 8, 0]
    leaf_k, internal_k, flags = struct.unpack('<HHI', b[16:24])
    assert (leaf_k, internal_k, flags) == (4, 16, 0)
    base, free, eof, driver = struct.unpack('<QQQQ', b[24:56])
    assert base == 0 and free == driver == 0xFFFFFFFFFFFFFFFF and eof == len(b)
    name_off, _, cache, _, btree, heap = struct.unpack('<QQIIQQ', b[56:96])
    assert name_off == 0 and cache == 1
    assert b[btree:btree + 4] == b'TREE' and b[heap:heap + 4] == b'HEAP'
    _, free_head, data = struct.unpack('<QQQ', b[heap + 8:heap + 32])
    assert free_head == 1 and b[data] == 0  # end-of-list marker; empty name at offset 0
    used = struct.unpack('<H', b[btree + 6:btree + 8])[0]
    snod = struct.unpack('<Q', b[btree + 32:btree + 40])[0]
    assert used == 1 and b[snod:snod + 8] == b'SNOD\x01\x00\x02\x00'
    assert h5._dtype_message('num', np.float32) == bytes.fromhex('11201f000400000000002000170800177f000000')
    assert h5._dtype_message('bool', None) == bytes.fromhex(
        '180200000100000010080000010000000000080046414c5345000000545255450000000000010000')[:38]


def _v3_file():
    """A superblock-v3 file by hand: root object header v2 whose link sits in a continuation
    block, a dataset with a v2 dataspace, compact layout and a v3 attribute holding a
    variable-length UTF-8 string in a global heap collection."""
    U = 0xFFFFFFFFFFFFFFFF

    def ohdr(msgs):
        body = b''.join(struct.pack('<BHB', t, len(d), 0) + d for t, d in msgs)
        return b'OHDR' + bytes([2, 0, len(body)]) + body + b'\0' * 4

    vals = np.array([1.5, -2.25, 3.0])
    f64 = struct.pack('<B3sIHHBBBBI', 0x11, bytes([0x20, 63, 0]), 8, 0, 64, 52, 11, 0, 52, 1023)
    text = 'café'.encode('utf-8')
    vstr = struct.pack('<B3sI', 0x19, bytes([0x01, 0x01, 0]), 16) + struct.pack('<B3sIHH', 0x10, b'\0\0\0', 1, 0, 8)
    name = b'unit\0'
    gcol_at = 512
    attr = struct.pack('<BBHHHB', 3, 0, len(name), len(vstr), 4, 0) + name + vstr + bytes([2, 0, 0, 0]) + \
        struct.pack('<IQI', len(text), gcol_at, 1)
    ds = ohdr([(0x01, bytes([2, 1, 0, 1]) + struct.pack('<Q', 3)), (0x03, f64),
               (0x08, struct.pack('<BBH', 3, 0, 24) + vals.tobytes()), (0x0C, attr)])
    ds_at = 256
    link = bytes([1, 0, 3]) + b'vel' + struct.pack('<Q', ds_at)
    ochk_at = 400
    ochk = b'OCHK' + struct.pack('<BHB', 0x06, len(link), 0) + link + b'\0' * 4
    root = ohdr([(0x10, struct.pack('<QQ', ochk_at, len(ochk)))])
    obj = struct.pack('<HHIQ', 1, 1, 0, len(text)) + text + b'\0' * ((-len(text)) % 8)
    gcol = b'GCOL' + bytes([1, 0, 0, 0]) + struct.pack('<Q', 16 + len(obj) + 16) + obj + b'\0' * 16
    buf = bytearray(1024)
    buf[0:48] = b'\x89HDF\r\n\x1a\n' + bytes([3, 8, 8, 0]) + struct.pack('<QQQQ', 0, U, 1024, 64) + b'\0' * 4
    buf[64:64 + len(root)] = root
    buf[ds_at:ds_at + len(ds)] = ds
    buf[ochk_at:ochk_at + len(ochk)] = ochk
    buf[gcol_at:gcol_at + len(gcol)] = gcol
    return bytes(buf), vals


def test_superblock_v3_object_header_v2_paths(tmp_path):
    data, vals = _v3_file()
    path = str(tmp_path / 'v3.h5')
    with open(path, 'wb') as fh:
        fh.write(data)
    root = h5.read_file(path)
    assert list(root.keys()) == ['vel']
    ds = root['vel']
    assert ds.shape == (3,) and np.array_equal(ds[()], vals)
    assert ds.attrs['unit'] == 'café'


def _dense_file(n):
    """A superblock-v3 file by hand whose root group keeps n links in dense storage: a link info
    message pointing at a fractal heap (root direct block of link messages) and at its v2 B-tree
    name index (one leaf of type-5 records: name hash, 7-byte managed heap ID)."""
    U = 0xFFFFFFFFFFFFFFFF
    buf = bytearray(8192)

    def ohdr(msgs):
        body = b''.join(struct.pack('<BHB', t, len(d), 0) + d for t, d in msgs)
        return b'OHDR' + bytes([2, 1]) + struct.pack('<H', len(body)) + body + b'\0' * 4

    f32 = struct.pack('<B3sIHHBBBBI', 0x11, bytes([0x20, 31, 0]), 4, 0, 32, 23, 8, 0, 23, 127)
    at, targets = 4096, []
    for k in range(n):  # scalar datasets holding k, compact layout
        ds = ohdr([(0x01, bytes([2, 0, 0, 0])), (0x03, f32), (0x08, struct.pack('<BBH', 3, 0, 4) +
                                                              np.float32(k).tobytes())])
        buf[at:at + len(ds)] = ds
        targets.append(at)
        at += (len(ds) + 7) // 8 * 8
    heap_at, block_at, tree_at, leaf_at = 1024, 1536, 2560, 3072
    objs, ids, off = b'', [], 17  # direct block header: 4 + 1 + 8 + 4 (offset bytes)
    for k in range(n):
        name = ('key%02d' % k).encode()
        link = bytes([1, 0, len(name)]) + name + struct.pack('<Q', targets[k])
        ids.append(bytes([0]) + struct.pack('<I', off) + struct.pack('<H', len(link)))
        objs += link
        off += len(link)
    block = b'FHDB' + bytes([0]) + struct.pack('<Q', heap_at) + struct.pack('<I', 0) + objs
    buf[block_at:block_at + len(block)] = block
    frhp = b'FRHP' + bytes([0]) + struct.pack('<HHBI', 7, 0, 0, 65536) + struct.pack('<QQQQ', 0, U, 0, U) + \
        struct.pack('<8Q', 512, 512, off, n, 0, 0, 0, 0) + struct.pack('<HQQHH', 4, 512, 65536, 32, 1) + \
        struct.pack('<QH', block_at, 0) + b'\0' * 4
    buf[heap_at:heap_at + len(frhp)] = frhp
    leaf = b'BTLF' + bytes([0, 5]) + b''.join(struct.pack('<I', 0) + i for i in ids) + b'\0' * 4
    buf[leaf_at:leaf_at + len(leaf)] = leaf
    bthd = b'BTHD' + bytes([0, 5]) + struct.pack('<IHHBB', 512, 11, 0, 100, 40) + struct.pack('<QHQ', leaf_at, n, n)
    buf[tree_at:tree_at + len(bthd) + 4] = bthd + b'\0' * 4
    root = ohdr([(0x02, bytes([0, 0]) + struct.pack('<QQ', heap_at, tree_at))])
    buf[64:64 + len(root)] = root
    buf[0:48] = b'\x89HDF\r\n\x1a\n' + bytes([3, 8, 8, 0]) + struct.pack('<QQQQ', 0, U, len(buf), 64) + b'\0' * 4
    return bytes(buf)


def test_dense_link_storage(tmp_path):
    path = str(tmp_path / 'dense.h5')
    with open(path, 'wb') as fh:
        fh.write(_dense_file(11))
    root = h5.read_file(path)
    assert sorted(root.keys()) == ['key%02d' % k for k in range(11)]
    assert all(root['key%02d' % k][()] == np.float32(k) for k in range(11))


def test_hard_link_cycle_is_an_error(tmp_path):
    """A group that links to itself (legal in HDF5) ends in ValueError, not unbounded recursion."""
    U = 0xFFFFFFFFFFFFFFFF
    link = bytes([1, 0, 4]) + b'self' + struct.pack('<Q', 64)
    body = struct.pack('<BHB', 0x06, len(link), 0) + link
    root = b'OHDR' + bytes([2, 0, len(body)]) + body + b'\0' * 4
    buf = bytearray(256)
    buf[0:48] = b'\x89HDF\r\n\x1a\n' + bytes([3, 8, 8, 0]) + struct.pack('<QQQQ', 0, U, 256, 64) + b'\0' * 4
    buf[64:64 + len(root)] = root
    path = str(tmp_path / 'cycle.h5')
    with open(path, 'wb') as fh:
        fh.write(bytes(buf))
    with pytest.raises(ValueError):
        h5.read_file(path)


def test_mosaic_file_naming_and_versions(tmp_path):
    p = str(tmp_path)
    kw = dict(project_name='breast', parameter='vp_model', path=p)
    with h5.HDF5(mode='w', **kw) as f:
        assert os.path.basename(f.filename) == 'breast-VpModel.h5'
        f.dump({'v': 0})
    with h5.HDF5(mode='w', **kw) as f:  # the next free version
        assert os.path.basename(f.filename) == 'breast-VpModel-00001.h5'
        f.dump({'v': 1})
    with h5.HDF5(mode='r', **kw) as f:  # the latest version
        assert f.load().v == 1
    assert h5.file_exists(version=1, **kw) and not h5.file_exists(version=2, **kw)
    with h5.HDF5(mode='r', version=0, **kw) as f:
        assert f.load().v == 0
    with h5.HDF5(mode='a', version=0, **kw) as f:
        f.append({'w': 'x'})
    got = h5.HDF5(mode='r', version=0, **kw).load()
    assert got.v == 0 and got.w == 'x'
    with pytest.raises(RuntimeError):
        h5.HDF5(mode='r', path=p)


def test_problem_model_dump_and_load(tmp_path):
    space = problem.Space((30, 34), 0.5e-3, extra=(6, 6), absorbing=(4, 4))
    time = problem.Time(0., 1e-7, 50)
    grid = problem.Grid(space, time)
    rng = np.random.default_rng(1)
    vp = problem.ScalarField('vp', grid, data=(1500 + 50 * rng.standard_normal(space.extended_shape)))
    vp.dump(project_name='p', path=str(tmp_path))
    back = problem.ScalarField('vp', grid)
    back.load(project_name='p', path=str(tmp_path))
    assert np.array_equal(back.data, vp.data)
    # the stored inner data padded with edge values, as StructuredData.pad_data does
    assert np.array_equal(back.extended_data, np.pad(vp.data, 6, mode='edge'))
    d = h5.HDF5(project_name='p', parameter='vp', path=str(tmp_path), mode='r').load(lazy=False)
    assert d.inner == [['6', '36', 'None'], ['6', '40', 'None']] and d.extended_shape == (42, 46)
    other = problem.ScalarField('vp', problem.Grid(problem.Space((10, 10), 0.5e-3), time))
    with pytest.raises(ValueError):
        other.load(project_name='p', path=str(tmp_path))
    tr = problem.Traces('observed', rng.standard_normal((5, 50)).astype(np.float32), grid)
    tr.dump(project_name='p', path=str(tmp_path))
    t2 = problem.Traces('observed', np.zeros((1, 1), np.float32))
    t2.load(project_name='p', path=str(tmp_path))
    assert np.array_equal(t2.data, tr.data)
    d = h5.HDF5(project_name='p', parameter='observed', path=str(tmp_path), mode='r').load(lazy=False)
    assert d.num_transducers == 5 and d.transducer_ids == [0, 1, 2, 3, 4] and d.time.num == 50


def test_unsupported_structures_raise(tmp_path):
    path = str(tmp_path / 'c.h5')
    with open(path, 'wb') as fh:
        fh.write(b'not hdf5' * 100)
    with pytest.raises(ValueError):
        h5.read_file(path)
    with pytest.raises(TypeError):
        h5.write_file(str(tmp_path / 'x.h5'), {'z': np.ones(2, np.complex64)})


def test_fwi_state_dump_and_restart(tmp_path):
    """The inversion's per-iteration dumps (model versions and loop records) and the restart
    from the latest or a chosen version, as the reference's optimisation loop keeps them."""
    rng = np.random.default_rng(4)
    vp = rng.uniform(1400, 1600, (40, 44)).astype(np.float32)
    inner = (slice(6, 34), slice(6, 38))
    hist = []
    models = []
    for k in range(3):
        models.append(vp + k)
        assert fwi.dump_state(models[-1], hist, inner, (5e-4, 5e-4), str(tmp_path), 'inv') == k
        hist.append({'misfit': 10.0 - k, 'error': 0.03 - 0.01 * k, 'seconds': 0.5, 'f_max': None if k else 3e5})
    assert sorted(os.listdir(tmp_path)) == ['inv-OptimisationLoop.h5', 'inv-Vp-00001.h5', 'inv-Vp-00002.h5',
                                            'inv-Vp.h5']
    v, h, done = fwi.load_state(str(tmp_path), 'inv')
    assert done == 2 and np.array_equal(v, models[2]) and h == hist[:2]
    v, h, done = fwi.load_state(str(tmp_path), 'inv', version=1)
    assert done == 1 and np.array_equal(v, models[1]) and h == hist[:1]
    # the model file is the reference's vp field description: inner data and grid
    d = h5.HDF5(project_name='inv', parameter='vp', path=str(tmp_path), version=2, mode='r').load(lazy=False)
    assert np.array_equal(d.data, models[2][inner]) and d.space.extra == (6, 6) and d.extended_shape == (40, 44)


def test_rewrite_keeps_a_live_mapping_readable(tmp_path):
    """A lazy dataset of an open file stays readable after the same file is appended to or dumped
    over: the writer replaces the file instead of truncating the mapped one."""
    fn = str(tmp_path / 'm.h5')
    data = np.arange(4096, dtype=np.float32).reshape(64, 64)
    h5.HDF5(fn, mode='w').dump({'data': data, 'name': 'a'})
    reader = h5.HDF5(fn, mode='r')
    lazy = reader.load(lazy=True)
    h5.HDF5(fn, mode='a').append({'extra': np.ones(3)})
    h5.HDF5(fn, mode='w').dump({'other': np.zeros(2)})
    np.testing.assert_array_equal(lazy['data'][()], data)  # the old file's contents
    reader.close()
    assert list(h5.HDF5(fn, mode='r').load(lazy=False).keys()) == ['other']
    assert oct(os.stat(fn).st_mode & 0o777) == oct(0o666 & ~_umask())


def _umask():
    m = os.umask(0)
    os.umask(m)
    return m


def test_close_behaviour(tmp_path):
    fn = str(tmp_path / 'c.h5')
    h5.HDF5(fn, mode='w').dump({'data': np.arange(10.)})
    f = h5.HDF5(fn, mode='r')
    lazy = f.load(lazy=True)
    f.close()
    with pytest.raises(ValueError, match='closed'):
        lazy['data'][()]
    f.close()  # a second close is a no-op
    # a non-lazy load through a writing handle reads everything and releases its mapping
    got = h5.HDF5(fn, mode='a').load(lazy=False)
    np.testing.assert_array_equal(got['data'], np.arange(10.))
    # an empty file: opening fails on the superblock, closing a File over no bytes is a no-op
    empty = str(tmp_path / 'empty.h5')
    open(empty, 'wb').close()
    with pytest.raises(Exception):
        h5.File(empty)
    obj = h5.File.__new__(h5.File)
    obj._b, obj.filename = b'', empty
    obj.close()
