"""The .h5 state files (io_state.py:30-85 of the reference) and restarts
(case_setup.py:184-194): the writer's structure against the HDF5 file format
specification (several symbol nodes under the root B-tree), round trips of
every field type a state holds, the reader on a file libhdf5 wrote, on
big-endian data, after a user block and on files it cannot read, the trajectory naming and the fluid-only state0 overwrite.
"""

import os
import struct

import numpy as np
import pytest
import torch

from jaxsph_gb300 import io_state as io


def state_like(n=257, dim=3, seed=0):
    g = torch.Generator().manual_seed(seed)
    return {
        "r": torch.rand((n, dim), generator=g),
        "u": torch.randn((n, dim), generator=g),
        "tag": torch.randint(0, 3, (n,), generator=g, dtype=torch.int32),
        "rho": torch.rand(n, generator=g).double(),
        "mass": torch.full((n,), 0.25),
        "step": np.int64(17),
        "flags": np.array([True, False, True]),
        "empty": np.zeros((0, dim), np.float32),
    }


def test_round_trip_of_state_fields(tmp_path):
    st = state_like()
    p = tmp_path / "s.h5"
    io.write_h5(st, str(p))
    back = io.read_h5(str(p), "numpy")
    assert sorted(back) == sorted(st)
    for k, v in st.items():
        want = v.numpy() if isinstance(v, torch.Tensor) else np.asarray(v)
        if want.dtype == np.bool_:
            want = want.astype(np.uint8)  # booleans are stored as uint8
        assert back[k].dtype == want.dtype and back[k].shape == want.shape, k
        assert np.array_equal(back[k], want), k
    t = io.read_h5(str(p))
    assert isinstance(t["r"], torch.Tensor) and torch.equal(t["r"], st["r"])
    with pytest.raises(ValueError):
        io.read_h5(str(p), "jax")


def test_writer_structure_follows_the_format_specification(tmp_path):
    p = tmp_path / "s.h5"
    io.write_h5({f"f{i:02d}": np.arange(i + 1, dtype=np.float32) for i in range(20)}, str(p))
    b = p.read_bytes()
    assert b[:8] == b"\x89HDF\r\n\x1a\n"
    assert b[8] == 0 and b[13] == 8 and b[14] == 8           # superblock v0, 8-byte sizes
    leaf_k, internal_k = struct.unpack_from("<HH", b, 16)
    base, free, eof, drv = struct.unpack_from("<QQQQ", b, 24)
    assert (leaf_k, internal_k, base) == (4, 16, 0)
    assert eof == len(b) and free == drv == 2 ** 64 - 1
    _, root_oh, cache = struct.unpack_from("<QQI", b, 56)
    btree, heap = struct.unpack_from("<QQ", b, 80)
    assert cache == 1 and b[root_oh] == 1
    assert b[heap:heap + 4] == b"HEAP" and b[btree:btree + 4] == b"TREE"
    # symbol table message of the root object header repeats the cached addresses
    mtype, msize = struct.unpack_from("<HH", b, root_oh + 16)
    assert (mtype, msize) == (0x0011, 16)
    assert struct.unpack_from("<QQ", b, root_oh + 24) == (btree, heap)
    # local heap: free list head is a real block whose next pointer is 1
    dsize, free_head, data_at = struct.unpack_from("<QQQ", b, heap + 8)
    nxt, fsize = struct.unpack_from("<QQ", b, data_at + free_head)
    assert nxt == 1 and free_head + fsize == dsize and free_head % 8 == 0
    # B-tree: 3 symbol nodes (8 + 8 + 4 names), keys = last name of each child
    ntype, level, used = struct.unpack_from("<BBH", b, btree + 4)
    assert (ntype, level, used) == (0, 0, 3)
    keys, kids = [], []
    q = btree + 24
    keys.append(struct.unpack_from("<Q", b, q)[0])
    for _ in range(used):
        child, key = struct.unpack_from("<QQ", b, q + 8)
        kids.append(child)
        keys.append(key)
        q += 16

    def name(off):
        s = data_at + off
        return b[s:b.index(b"\x00", s)].decode()

    assert keys[0] == 0 and [name(k) for k in keys[1:]] == ["f07", "f15", "f19"]
    seen = []
    for c in kids:
        assert b[c:c + 4] == b"SNOD" and b[c + 4] == 1
        (m,) = struct.unpack_from("<H", b, c + 6)
        assert m <= 8
        for e in range(m):
            off, oh = struct.unpack_from("<QQ", b, c + 8 + 40 * e)
            seen.append(name(off))
            # dataset object header: version 1, 8-aligned messages that fill it
            ver, _, nmsg, refc, size = struct.unpack_from("<BBHII", b, oh)
            assert (ver, refc, nmsg) == (1, 1, 4)
            pos, types = oh + 16, []
            while pos < oh + 16 + size:
                t, sz = struct.unpack_from("<HH", b, pos)
                assert sz % 8 == 0
                types.append(t)
                pos += 8 + sz
            assert pos == oh + 16 + size and types == [0x0001, 0x0003, 0x0005, 0x0008]
    assert seen == sorted(seen) and len(seen) == 20


def _find_datatype(b, oh):
    pos = oh + 16
    while True:
        t, sz = struct.unpack_from("<HH", b, pos)
        if t == 0x0003:
            return pos + 8
        pos += 8 + sz


def _data_address(b, oh):
    pos = oh + 16
    while True:
        t, sz = struct.unpack_from("<HH", b, pos)
        if t == 0x0008:
            return struct.unpack_from("<QQ", b, pos + 8 + 2)
        pos += 8 + sz


def test_reader_takes_big_endian_data(tmp_path):
    a = np.linspace(-3, 7, 11).astype(np.float32)
    p = tmp_path / "be.h5"
    io.write_h5({"x": a}, str(p))
    b = bytearray(p.read_bytes())
    (snod,) = struct.unpack_from("<Q", b, struct.unpack_from("<Q", b, 80)[0] + 32)
    (oh,) = struct.unpack_from("<Q", b, snod + 16)
    b[_find_datatype(b, oh) + 1] |= 1                    # byte order bit: big endian
    at, n = _data_address(b, oh)
    b[at:at + n] = a.astype(">f4").tobytes()
    p.write_bytes(bytes(b))
    back = io.read_h5(str(p), "numpy")["x"]
    assert back.dtype == np.float32 and np.array_equal(back, a)


def test_reader_takes_a_file_written_by_libhdf5(tmp_path):
    """An HDF5 file that libhdf5 itself wrote (MATLAB 7.3 format: a 512-byte
    user block, then a version-0 superblock; one float64 dataset with
    attribute messages the reader passes over), from scipy's test data."""
    scipy_io = pytest.importorskip("scipy.io")
    path = os.path.join(os.path.dirname(scipy_io.__file__), "matlab", "tests", "data",
                        "testhdf5_7.4_GLNX86.mat")
    if not os.path.exists(path):
        pytest.skip("scipy's test data is not installed")
    back = io.read_h5(path, "numpy")
    assert list(back) == ["testdouble"]
    x = back["testdouble"]
    assert x.dtype == np.float64 and x.shape == (9, 1)
    assert np.allclose(x[:, 0], np.arange(9) * np.pi / 4, rtol=0, atol=1e-15)
    # the writer encodes the same array's dataspace and datatype messages
    # byte for byte as libhdf5 did
    mine = tmp_path / "mine.h5"
    io.write_h5({"testdouble": x}, str(mine))

    def messages(file_name):
        f = io._File(open(file_name, "rb").read())
        e = f.root
        (entry,) = f.group_entries(f.off(e + f.sl + f.so + 8), f.off(e + f.sl + f.so + 16))
        return {t: bytes(d) for t, d in f.messages(entry[1])}

    theirs, ours = messages(path), messages(str(mine))
    for mtype in (0x0001, 0x0003):                 # dataspace, datatype
        assert ours[mtype] == theirs[mtype], hex(mtype)

    def group(file_name):
        """Root group fields that do not depend on sizes or addresses."""
        b = open(file_name, "rb").read()
        f = io._File(b)
        e = f.root
        cache = f.uint(e + 16, 4)
        bt, hp = f.addr(f.off(e + 24)), f.addr(f.off(e + 32))
        dsize, free, data = struct.unpack_from("<QQQ", b, hp + 8)
        nxt, fsize = struct.unpack_from("<QQ", b, f.addr(data) + free)
        node = struct.unpack_from("<4sBBHQQQ", b, bt)   # sig, type, level, used, left, right, key0
        child, key1 = struct.unpack_from("<QQ", b, bt + 32)
        snod = struct.unpack_from("<4sBBH", b, f.addr(child))
        entry = struct.unpack_from("<QQI", b, f.addr(child) + 8)
        return (cache, b[hp:hp + 8], free, nxt, free + fsize == dsize, node, key1, snod,
                entry[0], entry[2])

    assert group(str(mine)) == group(path)


def test_reader_finds_the_superblock_after_a_user_block(tmp_path):
    a = np.arange(12, dtype=np.int32).reshape(3, 4)
    p = tmp_path / "s.h5"
    io.write_h5({"a": a}, str(p))
    b = bytearray(p.read_bytes())
    for ub in (512, 2048):
        q = bytearray(b"u" * ub) + b
        struct.pack_into("<Q", q, ub + 24, ub)          # base address: the superblock
        p.write_bytes(bytes(q))
        assert np.array_equal(io.read_h5(str(p), "numpy")["a"], a)


def test_reader_rejects_what_it_does_not_read(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not hdf5" * 4)
    with pytest.raises(ValueError, match="not an HDF5 file"):
        io.read_h5(str(p))
    io.write_h5({"x": np.zeros(3, np.float32)}, str(p))
    b = bytearray(p.read_bytes())
    b[8] = 2                                             # superblock version 2
    p.write_bytes(bytes(b))
    with pytest.raises(ValueError, match="superblock version 2"):
        io.read_h5(str(p))
    with pytest.raises(TypeError):
        io.write_h5({"c": np.zeros(2, np.complex64)}, str(p))


def test_write_state_names_files_like_the_reference(tmp_path):
    st = {"r": np.zeros((2, 2), np.float32)}
    got = [io.write_state(k, st, str(tmp_path), 250, write_every=50) for k in range(-1, 251)]
    names = sorted(os.path.basename(x) for x in got if x)
    assert names == [f"traj_{k:03d}.h5" for k in range(0, 251, 50)]
    assert io.write_state(249, st, str(tmp_path), 250, mode="rlx", name="tgv_2_0.02_42")
    assert io.write_state(248, st, str(tmp_path), 250, mode="rlx", name="x") is None
    assert (tmp_path / "tgv_2_0.02_42.h5").exists()


def test_state0_overwrites_fluid_particles_only(tmp_path):
    from jaxsph_gb300 import cases

    setup = cases.lid_driven_cavity(dx=0.1)
    saved = {k: v.clone() for k, v in setup.state.items()}
    fluid = saved["tag"] == 0
    saved["r"][fluid] += 0.01
    saved["u"][fluid] = 0.5
    p = tmp_path / "state0.h5"
    io.write_h5(saved, str(p))
    before = {k: v.clone() for k, v in setup.state.items()}
    setup.load_state0(str(p), keys=("r", "u"))
    assert torch.equal(setup.state["r"], saved["r"])
    assert torch.equal(setup.state["u"][fluid], saved["u"][fluid])
    assert torch.equal(setup.state["u"][~fluid], before["u"][~fluid])
    assert torch.equal(setup.state["rho"], before["rho"])
    with pytest.raises(ValueError, match="not found"):
        io.write_h5({"tag": saved["tag"]}, str(p))
        setup.load_state0(str(p), keys=("r",))
    keep = torch.ones_like(fluid)
    keep[torch.nonzero(fluid).squeeze(1)[:9]] = False     # nine fluid particles fewer
    io.write_h5({"tag": saved["tag"][keep], "r": saved["r"][keep]}, str(p))
    with pytest.raises(ValueError, match="Shape mismatch"):
        setup.load_state0(str(p), keys=("r",))
