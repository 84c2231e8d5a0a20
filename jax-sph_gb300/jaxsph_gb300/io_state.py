"""State input/output in the reference's ``.h5`` trajectory format
(``jax_sph/io_state.py:30-85``) and restarts from a saved state
(``case_setup.py:184-194``).

The reference writes one HDF5 file per saved step with h5py, one dataset per
state field in the root group (``write_h5``), and reads them back with
``read_h5``. Neither h5py nor libhdf5 is needed here: this module writes and
reads the subset of the HDF5 format such files use, as the HDF5 file format
specification defines it --

* superblock version 0 or 1, 8- or 4-byte offsets and lengths, at offset 0
  or after a user block (offset 512, 1024, 2048, ...);
* the root group as a symbol table (version-1 B-tree of symbol nodes, names
  in a local heap);
* version-1 object headers (with continuation blocks) holding a dataspace
  (version 1 or 2), an integer or IEEE float datatype of either byte order
  (and h5py's boolean enum), and a contiguous or compact data layout
  (version 3 or 4; older layouts are read for contiguous data).

The writer emits exactly that structure, in the form libhdf5 itself writes
for ``h5py.File(path, "w").create_dataset(name, data=array)`` with default
settings. Files with newer superblocks (``libver="latest"``), chunked or
compressed datasets, or nested groups are rejected with an error naming the
unsupported feature. Booleans are written as uint8.
"""

import os
import struct

import numpy as np
import torch

__all__ = ["write_h5", "read_h5", "write_state", "apply_state0"]

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF
_LEAF_K, _INTERNAL_K = 4, 16          # group leaf / internal node K (libhdf5 defaults)
_SNOD_SIZE = 8 + 2 * _LEAF_K * 40     # symbol table node, allocated full
_TREE_SIZE = 24 + 2 * _INTERNAL_K * 8 + (2 * _INTERNAL_K + 1) * 8


def _pad8(n):
    return (n + 7) & ~7


# ------------------------------------------------------------------ datatypes
def _dtype_message(dt):
    """Datatype message (type 0x0003, version 1) of a numpy dtype."""
    dt = np.dtype(dt).newbyteorder("<") if np.dtype(dt).byteorder == ">" else np.dtype(dt)
    size = dt.itemsize
    if dt.kind in "iu":
        bits = 0x08 if dt.kind == "i" else 0x00
        head = struct.pack("<B3BI", 0x10 | 0, bits, 0, 0, size)
        return head + struct.pack("<HH", 0, 8 * size)
    if dt.kind == "f" and size in (2, 4, 8):
        exp_size, mant_size, bias = {2: (5, 10, 15), 4: (8, 23, 127), 8: (11, 52, 1023)}[size]
        sign = 8 * size - 1
        head = struct.pack("<B3BI", 0x10 | 1, 0x20, sign, 0, size)
        return head + struct.pack("<HHBBBBI", 0, 8 * size, mant_size, exp_size, 0, mant_size,
                                  bias)
    raise TypeError(f"dtype {dt} has no HDF5 integer/float encoding here")


def _parse_dtype(b):
    cls_ver, f0, f1, f2, size = struct.unpack_from("<B3BI", b, 0)
    cls = cls_ver & 0x0F
    order = ">" if f0 & 1 else "<"
    if cls == 0:
        signed = bool(f0 & 0x08)
        if size not in (1, 2, 4, 8):
            raise ValueError(f"integer datatype of {size} bytes")
        return np.dtype(f"{order}{'i' if signed else 'u'}{size}")
    if cls == 1:
        if size not in (2, 4, 8):
            raise ValueError(f"float datatype of {size} bytes")
        return np.dtype(f"{order}f{size}")
    if cls == 8 and size == 1:  # h5py's numpy bool: an enum over int8
        return np.dtype(np.bool_)
    raise ValueError(f"HDF5 datatype class {cls} is not supported")


# ------------------------------------------------------------------ writer
def _as_numpy(v):
    if isinstance(v, torch.Tensor):
        v = v.detach().cpu().numpy()
    a = np.asarray(v)
    if not a.flags.c_contiguous:
        a = a.copy(order="C")  # (ascontiguousarray would make a scalar 1-d)
    if a.dtype == np.bool_:
        a = a.astype(np.uint8)
    return a


def _message(mtype, data, flags=0):
    data = data + b"\x00" * (_pad8(len(data)) - len(data))
    return struct.pack("<HHB3x", mtype, len(data), flags) + data


def _object_header(messages):
    body = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body


def write_h5(data_dict, path):
    """Write a dict of arrays (numpy or torch) to an .h5 file, one dataset
    per key in the root group (io_state.py:30-35)."""
    items = sorted((str(k), _as_numpy(v)) for k, v in data_dict.items())
    names = [k for k, _ in items]
    if len(set(names)) != len(names):
        raise ValueError("duplicate dataset names")
    n_snod = max(1, -(-len(items) // (2 * _LEAF_K)))
    if n_snod > 2 * _INTERNAL_K:
        raise ValueError(f"at most {4 * _LEAF_K * _INTERNAL_K} datasets per file")

    # local heap data: "" at offset 0, then the names, then one free block
    heap = bytearray(8)
    name_off = {}
    for k in names:
        raw = k.encode("utf-8")
        if b"\x00" in raw or not raw:
            raise ValueError(f"invalid dataset name {k!r}")
        name_off[k] = len(heap)
        heap += raw + b"\x00" * (_pad8(len(raw) + 1) - len(raw))
    free_at = len(heap)
    heap += struct.pack("<QQ", 1, 16)   # last free block (next = 1), 16 bytes

    # dataset object headers without their data addresses: sizes first
    def dset_header(a, addr):
        shape = a.shape
        space = struct.pack("<BBB5x", 1, len(shape), 0) + b"".join(
            struct.pack("<Q", d) for d in shape)
        nbytes = a.nbytes
        layout = struct.pack("<BBQQ", 3, 1, addr if nbytes else _UNDEF, nbytes)
        fill = struct.pack("<BBBB", 2, 2, 2, 0)
        return _object_header([_message(0x0001, space), _message(0x0003, _dtype_message(a.dtype), 1),
                               _message(0x0005, fill, 1), _message(0x0008, layout)])

    sb_size = 96
    root_oh = _object_header([_message(0x0011, b"\x00" * 16)])
    a_root = sb_size
    a_heap = a_root + len(root_oh)
    a_heapdata = a_heap + 32
    a_tree = a_heapdata + len(heap)
    a_snod = a_tree + _TREE_SIZE
    a_dset = a_snod + n_snod * _SNOD_SIZE
    hdr_sizes = [len(dset_header(a, 0)) for _, a in items]
    a_data = a_dset + sum(hdr_sizes)
    dset_addr, data_addr, pos, dpos = [], [], a_dset, a_data
    for (_, a), hs in zip(items, hdr_sizes):
        dset_addr.append(pos)
        pos += hs
        data_addr.append(dpos)
        dpos += _pad8(a.nbytes)
    eof = dpos

    out = bytearray()
    # superblock version 0
    out += _SIG + struct.pack("<8B", 0, 0, 0, 0, 0, 8, 8, 0)
    out += struct.pack("<HHI", _LEAF_K, _INTERNAL_K, 0)
    out += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
    out += struct.pack("<QQI4xQQ", 0, a_root, 1, a_tree, a_heap)
    assert len(out) == sb_size
    out += _object_header([_message(0x0011, struct.pack("<QQ", a_tree, a_heap))])
    out += b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), free_at, a_heapdata)
    out += heap
    # one B-tree node (level 0) over the symbol nodes
    groups = [names[i:i + 2 * _LEAF_K] for i in range(0, len(names), 2 * _LEAF_K)] or [[]]
    tree = bytearray(b"TREE" + struct.pack("<BBHQQ", 0, 0, len(groups) if names else 0,
                                           _UNDEF, _UNDEF))
    tree += struct.pack("<Q", 0)
    for gi, g in enumerate(groups if names else []):
        tree += struct.pack("<QQ", a_snod + gi * _SNOD_SIZE, name_off[g[-1]])
    tree += b"\x00" * (_TREE_SIZE - len(tree))
    out += tree
    where = dict(zip(names, dset_addr))
    for g in groups:
        node = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, len(g)))
        for k in g:
            node += struct.pack("<QQI4x16x", name_off[k], where[k], 0)
        node += b"\x00" * (_SNOD_SIZE - len(node))
        out += node
    for (_, a), da in zip(items, data_addr):
        out += dset_header(a, da)
    assert len(out) == a_data
    for _, a in items:
        raw = a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
        out += raw + b"\x00" * (_pad8(len(raw)) - len(raw))
    assert len(out) == eof
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "wb") as f:
        f.write(out)
    os.replace(tmp, path)


# ------------------------------------------------------------------ reader
class _File:
    def __init__(self, buf):
        self.b = buf
        # the superblock starts at 0 or, after a user block, at 512 * 2^k;
        # its base address is absolute and every other address is relative
        # to it
        sb = 0
        while buf[sb:sb + 8] != _SIG:
            sb = 512 if sb == 0 else 2 * sb
            if sb + 8 > len(buf):
                raise ValueError("not an HDF5 file (no signature at offset 0, 512, 1024, ...)")
        ver = buf[sb + 8]
        if ver not in (0, 1):
            raise ValueError(f"HDF5 superblock version {ver} (libver='latest') is not supported")
        self.so, self.sl = buf[sb + 13], buf[sb + 14]
        if self.so not in (4, 8) or self.sl not in (4, 8):
            raise ValueError("unsupported HDF5 offset/length sizes")
        p = sb + 24 + (4 if ver == 1 else 0)
        self.base = self.off(p)
        p += 4 * self.so
        self.root = p   # root group symbol table entry

    def uint(self, p, n):
        return int.from_bytes(self.b[p:p + n], "little")

    def off(self, p):
        return self.uint(p, self.so)

    def ln(self, p):
        return self.uint(p, self.sl)

    def undef(self, a):
        return a == (1 << (8 * self.so)) - 1

    def addr(self, a):
        return self.base + a

    # version-1 object header -> list of (type, data)
    def messages(self, a):
        p = self.addr(a)
        if self.b[p] != 1:
            raise ValueError(f"object header version {self.b[p]} is not supported")
        nmsg = self.uint(p + 2, 2)
        size = self.uint(p + 8, 4)
        blocks, out = [(p + 16, size)], []
        while blocks and len(out) < nmsg:
            q, n = blocks.pop(0)
            end = q + n
            while q + 8 <= end and len(out) < nmsg:
                t, sz = self.uint(q, 2), self.uint(q + 2, 2)
                data = self.b[q + 8:q + 8 + sz]
                if t == 0x0010:  # continuation
                    blocks.append((self.addr(self.off(q + 8)), self.ln(q + 8 + self.so)))
                out.append((t, data))
                q += 8 + sz
        return out

    def heap_data(self, a):
        p = self.addr(a)
        if self.b[p:p + 4] != b"HEAP":
            raise ValueError("bad local heap")
        q = p + 8
        size = self.ln(q)
        data_at = self.off(q + 2 * self.sl)
        return self.addr(data_at), size

    def name(self, heap, off):
        start = heap[0] + off
        end = self.b.index(b"\x00", start)
        return self.b[start:end].decode("utf-8")

    def group_entries(self, btree, heap_addr):
        heap = self.heap_data(heap_addr)
        out = []

        def walk(a):
            p = self.addr(a)
            if self.b[p:p + 4] != b"TREE" or self.b[p + 4] != 0:
                raise ValueError("bad group B-tree node")
            level, n = self.b[p + 5], self.uint(p + 6, 2)
            q = p + 8 + 2 * self.so + self.sl       # first child after key 0
            for _ in range(n):
                child = self.off(q)
                if level > 0:
                    walk(child)
                else:
                    s = self.addr(child)
                    if self.b[s:s + 4] != b"SNOD":
                        raise ValueError("bad symbol table node")
                    m = self.uint(s + 6, 2)
                    e = s + 8
                    for _ in range(m):
                        out.append((self.name(heap, self.ln(e)), self.off(e + self.sl),
                                    self.uint(e + self.sl + self.so, 4)))
                        e += self.sl + self.so + 24
                q += self.so + self.sl

        walk(btree)
        return out

    def dataset(self, a):
        shape = dtype = None
        layout = None
        for t, d in self.messages(a):
            if t == 0x0001:
                ver, rank = d[0], d[1]
                if ver == 2 and d[3] == 2:
                    raise ValueError("null dataspaces are not supported")
                start = 8 if ver == 1 else 4
                shape = tuple(int.from_bytes(d[start + i * self.sl:start + (i + 1) * self.sl],
                                             "little") for i in range(rank))
            elif t == 0x0003:
                dtype = _parse_dtype(d)
            elif t == 0x0008:
                layout = d
            elif t == 0x0011:
                raise ValueError("nested groups are not supported")
        if shape is None or dtype is None or layout is None:
            raise ValueError("object is not a dataset")
        count = int(np.prod(shape)) if shape else 1
        ver = layout[0]
        if ver in (3, 4):
            cls = layout[1]
            if cls == 0:        # compact
                n = int.from_bytes(layout[2:4], "little")
                raw = bytes(layout[4:4 + n])
            elif cls == 1:      # contiguous
                at = int.from_bytes(layout[2:2 + self.so], "little")
                n = int.from_bytes(layout[2 + self.so:2 + self.so + self.sl], "little")
                raw = b"" if self.undef(at) else bytes(self.b[self.addr(at):self.addr(at) + n])
            else:
                raise ValueError("chunked or virtual datasets are not supported")
        elif ver in (1, 2):
            rank, cls = layout[1], layout[2]
            if cls != 1:
                raise ValueError("only contiguous data is supported in layout version 1/2")
            at = int.from_bytes(layout[8:8 + self.so], "little")
            n = count * dtype.itemsize
            raw = b"" if self.undef(at) else bytes(self.b[self.addr(at):self.addr(at) + n])
        else:
            raise ValueError(f"layout message version {ver} is not supported")
        need = count * dtype.itemsize
        if len(raw) < need:
            raw = raw + b"\x00" * (need - len(raw))  # never written: the fill value 0
        if dtype == np.bool_:
            return np.frombuffer(raw[:need], dtype=np.int8).reshape(shape) != 0
        return np.frombuffer(raw[:need], dtype=dtype).reshape(shape).astype(
            dtype.newbyteorder("="))


def read_h5(file_name, array_type="torch"):
    """Read an .h5 file into a dict of torch tensors or numpy arrays
    (io_state.py:69-85)."""
    if array_type not in ("torch", "numpy"):
        raise ValueError('array_type must be either "torch" or "numpy"')
    with open(file_name, "rb") as f:
        f_ = _File(f.read())
    e = f_.root
    cache = f_.uint(e + f_.sl + f_.so, 4)
    oh = f_.off(e + f_.sl)
    btree = heap = None
    if cache == 1:
        s = e + f_.sl + f_.so + 8
        btree, heap = f_.off(s), f_.off(s + f_.so)
    else:
        for t, d in f_.messages(oh):
            if t == 0x0011:
                btree = int.from_bytes(d[:f_.so], "little")
                heap = int.from_bytes(d[f_.so:2 * f_.so], "little")
    if btree is None:
        raise ValueError("root group has no symbol table (newer group format)")
    out = {}
    for name, addr, _ in sorted(f_.group_entries(btree, heap)):
        a = f_.dataset(addr)
        out[name] = torch.from_numpy(a.copy()) if array_type == "torch" else a
    return out


# ------------------------------------------------------------------ trajectories
def write_state(step, state, dir, sequence_length, write_every=1, mode="sim", name=None):
    """Write ``traj_<step>.h5`` every ``write_every`` steps (io_state.py:44-66):
    the step zero-padded to the digits of ``sequence_length``; in relaxation
    mode (``mode="rlx"``) only the last step, as ``<name>.h5``."""
    write_normal = mode == "sim" and step % write_every == 0 and step >= 0
    write_relax = mode == "rlx" and step == sequence_length - 1
    if not (write_normal or write_relax):
        return None
    if mode == "rlx":
        fname = name
    else:
        fname = "traj_" + str(step).zfill(len(str(sequence_length)))
    path = os.path.join(dir, fname + ".h5")
    write_h5(state, path)
    return path


def apply_state0(state, path, keys=("r",), fluid_tag=0):
    """Overwrite the fluid particles' ``keys`` of ``state`` with those of a
    saved state (case_setup.py:184-194): the fluid particles of both, in
    order, must match in number. Restart a run with every key."""
    saved = read_h5(path, "torch")
    for k in keys:
        if k not in state:
            continue
        if k not in saved:
            raise ValueError(f"Key {k} not found in state0 file.")
        mask = state["tag"] == fluid_tag
        smask = saved["tag"].to(state["tag"].device) == fluid_tag
        src = saved[k].to(state[k].device)[smask]
        if state[k][mask].shape != src.shape:
            raise ValueError(f"Shape mismatch for key {k} in state0 file.")
        state[k] = state[k].clone()
        state[k][mask] = src.to(state[k].dtype)
    return state
