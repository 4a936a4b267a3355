"""A minimal reader of the HDF5 files that netCDF-4 writes, for the reference's archived
Fortran outputs (fortran/monki/upstream/OUTPUT/testrun/*.nc).

Test infrastructure only: neither the product package nor the kernels import it. It is
written from the published HDF5 File Format Specification (version 3.0) and covers what
those files use: superblock versions 2 and 3, version 2 object headers with continuation
blocks, groups whose links are either link messages in the header or "dense" (a fractal
heap of link messages indexed by a version 2 B-tree of name hashes), and datasets of
fixed-point, floating-point or fixed-length string elements with compact, contiguous or
chunked (version 1 B-tree, deflate and shuffle filters) layout. Anything else raises
``NotImplementedError`` naming the structure.

    with HDF5File(path) as f:
        f.names()                 # the root group's link names
        f.read("std_radiance")    # numpy array in the file's (C) dimension order
        f.attributes("radiance")  # {"long_name": ..., "units": ..., ...}
"""

from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEFINED = 0xFFFFFFFFFFFFFFFF

# Object header message types used here (specification section IV.A.2).
DATASPACE, LINK_INFO, DATATYPE, LINK, LAYOUT, FILTERS, ATTRIBUTE, CONTINUATION = 0x01, 0x02, 0x03, 0x06, 0x08, 0x0B, 0x0C, 0x10


class HDF5File:
    def __init__(self, path):
        self.path = Path(path)
        self.data = self.path.read_bytes()
        if self.data[:8] != SIGNATURE:
            raise ValueError(f"{path} is not an HDF5 file")
        version = self.data[8]
        if version not in (2, 3):
            raise NotImplementedError(f"superblock version {version}")
        self.offset_size, self.length_size = self.data[9], self.data[10]
        if (self.offset_size, self.length_size) != (8, 8):
            raise NotImplementedError("offsets and lengths other than 8 bytes")
        # base address, superblock extension, end of file, root group object header
        self.base, _, _, self.root = struct.unpack_from("<4Q", self.data, 12)
        self._links = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    # ------------------------------------------------------------------ primitives
    def _u(self, at: int, size: int) -> int:
        return int.from_bytes(self.data[at : at + size], "little")

    def _address(self, at: int) -> int:
        return self._u(at, 8) + (0 if self._u(at, 8) == UNDEFINED else self.base)

    # ------------------------------------------------------------------ object headers
    def messages(self, address: int):
        """(type, body offset, body size) of every message of a version 2 object header,
        its continuation blocks included."""

        at = address
        if self.data[at : at + 4] != b"OHDR":
            raise NotImplementedError(f"object header at {address:#x} is not version 2")
        if self.data[at + 4] != 2:
            raise NotImplementedError("object header version")
        flags = self.data[at + 5]
        at += 6
        if flags & 0x20:
            at += 16  # access, modification, change and birth times
        if flags & 0x10:
            at += 4  # attribute storage phase change values
        width = 1 << (flags & 0x03)
        size = self._u(at, width)
        at += width
        order = 2 if flags & 0x04 else 0
        blocks = [(at, at + size)]
        found = []
        while blocks:
            start, end = blocks.pop(0)
            p = start
            while p + 4 + order <= end:
                kind, length = self.data[p], self._u(p + 1, 2)
                body = p + 4 + order
                if body + length > end:
                    break
                found.append((kind, body, length))
                if kind == CONTINUATION:
                    block, block_size = self._address(body), self._u(body + 8, 8)
                    if self.data[block : block + 4] != b"OCHK":
                        raise ValueError("object header continuation block signature")
                    blocks.append((block + 4, block + block_size - 4))
                p = body + length
        return found

    # ------------------------------------------------------------------ groups
    def links(self) -> dict:
        """Root group: link name -> object header address."""

        if self._links is None:
            self._links = {}
            for kind, body, _ in self.messages(self.root):
                if kind == LINK:
                    name, address = self._link(body)
                    self._links[name] = address
                elif kind == LINK_INFO:
                    self._dense_links(body)
        return self._links

    def names(self) -> list:
        return sorted(self.links())

    def _link(self, at: int):
        if self.data[at] != 1:
            raise NotImplementedError("link message version")
        flags = self.data[at + 1]
        p = at + 2
        link_type = 0
        if flags & 0x08:
            link_type = self.data[p]
            p += 1
        if flags & 0x04:
            p += 8  # creation order
        if flags & 0x10:
            p += 1  # name character set
        width = 1 << (flags & 0x03)
        length = self._u(p, width)
        p += width
        name = self.data[p : p + length].decode("utf-8")
        p += length
        if link_type != 0:
            return name, None  # soft or external link: not followed
        return name, self._address(p)

    def _dense_links(self, at: int):
        if self.data[at] != 0:
            raise NotImplementedError("link info message version")
        flags = self.data[at + 1]
        p = at + 2 + (8 if flags & 0x01 else 0)
        heap, index = self._address(p), self._address(p + 8)
        if heap == UNDEFINED or index == UNDEFINED:
            return
        fractal = FractalHeap(self, heap)
        for record in self._btree2_records(index):
            # Type 5 record (link name of an indexed group): name hash, heap ID.
            name, address = self._link(fractal.locate(record[4:]))
            self._links[name] = address

    def _btree2_records(self, address: int):
        if self.data[address : address + 4] != b"BTHD":
            raise ValueError("version 2 B-tree header signature")
        node_size = self._u(address + 6, 4)
        record_size = self._u(address + 10, 2)
        depth = self._u(address + 12, 2)
        root = self._address(address + 16)
        root_records = self._u(address + 24, 2)
        return list(self._btree2_node(root, root_records, depth, node_size, record_size))

    def _btree2_node(self, address, count, depth, node_size, record_size):
        if depth == 0:
            if self.data[address : address + 4] != b"BTLF":
                raise ValueError("version 2 B-tree leaf signature")
            p = address + 6
            for _ in range(count):
                yield self.data[p : p + record_size]
                p += record_size
            return
        if depth > 1:
            raise NotImplementedError("version 2 B-trees deeper than one internal level")
        if self.data[address : address + 4] != b"BTIN":
            raise ValueError("version 2 B-tree internal node signature")
        # Children of a depth-1 node are leaves; their record counts are stored in the
        # fewest bytes that hold the most records a leaf can have.
        leaf_max = (node_size - 10) // record_size
        width = max(1, (leaf_max.bit_length() + 7) // 8)
        p = address + 6
        records = []
        for _ in range(count):
            records.append(self.data[p : p + record_size])
            p += record_size
        for child in range(count + 1):
            child_address, child_count = self._address(p), self._u(p + 8, width)
            p += 8 + width
            yield from self._btree2_node(child_address, child_count, 0, node_size, record_size)
            if child < count:
                yield records[child]

    # ------------------------------------------------------------------ datasets
    def dataset(self, name: str) -> dict:
        address = self.links().get(name)
        if address is None:
            raise KeyError(name)
        info = {"shape": (), "filters": []}
        for kind, body, size in self.messages(address):
            if kind == DATASPACE:
                info["shape"] = self._dataspace(body)
            elif kind == DATATYPE:
                info["dtype"] = self._datatype(body)
            elif kind == LAYOUT:
                info["layout"] = self._layout(body, size)
            elif kind == FILTERS:
                info["filters"] = self._filters(body)
        return info

    def attributes(self, name: str) -> dict:
        """Attributes stored in a dataset's object header (compact storage): fixed-length
        strings as str, numbers as arrays. Attributes in dense storage are not read."""

        address = self.links().get(name)
        if address is None:
            raise KeyError(name)
        out = {}
        for kind, body, _ in self.messages(address):
            if kind != ATTRIBUTE:
                continue
            version = self.data[body]
            name_size, type_size, space_size = self._u(body + 2, 2), self._u(body + 4, 2), self._u(body + 6, 2)
            if version == 1:
                pad = lambda n: (n + 7) // 8 * 8  # noqa: E731
                p = body + 8
                key = self.data[p : p + name_size].split(b"\0")[0].decode()
                p += pad(name_size)
                dtype_at, p = p, p + pad(type_size)
                space_at, p = p, p + pad(space_size)
            elif version in (2, 3):
                p = body + 8 + (1 if version == 3 else 0)
                key = self.data[p : p + name_size].split(b"\0")[0].decode()
                p += name_size
                dtype_at, p = p, p + type_size
                space_at, p = p, p + space_size
            else:
                raise NotImplementedError(f"attribute message version {version}")
            cls = self.data[dtype_at] & 0x0F
            if cls not in (0, 1, 3):
                continue  # references and variable-length data (netCDF-4 bookkeeping)
            dtype = self._datatype(dtype_at)
            shape = self._dataspace(space_at)
            count = int(np.prod(shape)) if shape else 1
            raw = self.data[p : p + count * dtype.itemsize]
            if cls == 3:
                out[key] = b"".join(np.frombuffer(raw, dtype=dtype)).split(b"\0")[0].decode("utf-8", "replace")
            else:
                out[key] = np.frombuffer(raw, dtype=dtype).copy()
        return out

    def read(self, name: str) -> np.ndarray:
        info = self.dataset(name)
        shape, dtype = info["shape"], info["dtype"]
        count = int(np.prod(shape)) if shape else 1
        layout = info["layout"]
        if layout[0] == "compact":
            raw = layout[1]
        elif layout[0] == "contiguous":
            start, size = layout[1], layout[2]
            raw = self.data[start : start + size] if start != UNDEFINED else bytes(count * dtype.itemsize)
        else:
            raw = self._chunked(layout, shape, dtype, info["filters"])
        values = np.frombuffer(raw[: count * dtype.itemsize], dtype=dtype).copy()
        if values.size != count:
            raise ValueError(f"{name}: {values.size} elements for shape {shape}")
        return values.reshape(shape) if shape else values[0]

    def _dataspace(self, at: int):
        version, rank, flags = self.data[at], self.data[at + 1], self.data[at + 2]
        if version == 1:
            p = at + 8
        elif version == 2:
            if self.data[at + 3] == 0:  # scalar
                return ()
            p = at + 4
        else:
            raise NotImplementedError("dataspace version")
        return tuple(self._u(p + 8 * d, 8) for d in range(rank))

    def _datatype(self, at: int):
        cls = self.data[at] & 0x0F
        bits = self.data[at + 1]
        size = self._u(at + 4, 4)
        order = ">" if bits & 0x01 else "<"
        if cls == 0:
            return np.dtype(f"{order}{'i' if bits & 0x08 else 'u'}{size}")
        if cls == 1:
            return np.dtype(f"{order}f{size}")
        if cls == 3:
            return np.dtype(f"S{size}")
        raise NotImplementedError(f"datatype class {cls}")

    def _layout(self, at: int, size: int):
        version, cls = self.data[at], self.data[at + 1]
        if version != 3:
            raise NotImplementedError(f"data layout message version {version}")
        if cls == 0:
            n = self._u(at + 2, 2)
            return ("compact", self.data[at + 4 : at + 4 + n])
        if cls == 1:
            return ("contiguous", self._address(at + 2), self._u(at + 10, 8))
        if cls == 2:
            rank = self.data[at + 2]  # dataset rank + 1: the last chunk dimension is the element size
            btree = self._address(at + 3)
            dims = tuple(self._u(at + 11 + 4 * d, 4) for d in range(rank))
            return ("chunked", btree, dims)
        raise NotImplementedError(f"layout class {cls}")

    def _filters(self, at: int):
        version, count = self.data[at], self.data[at + 1]
        p = at + (8 if version == 1 else 2)
        out = []
        for _ in range(count):
            ident = self._u(p, 2)
            name_length = self._u(p + 2, 2) if (version == 1 or ident >= 256) else 0
            values = self._u(p + 6, 2) if (version == 1 or ident >= 256) else self._u(p + 4, 2)
            p += 8 if (version == 1 or ident >= 256) else 6
            if version == 1:
                p += (name_length + 7) // 8 * 8
            else:
                p += name_length
            client = [self._u(p + 4 * v, 4) for v in range(values)]
            p += 4 * values
            if version == 1 and values % 2:
                p += 4
            out.append((ident, client))
        return out

    def _chunked(self, layout, shape, dtype, filters):
        _, btree, dims = layout
        chunk = dims[:-1]
        out = np.zeros(shape, dtype=dtype)
        for offsets, raw, mask in self._chunks(btree, len(chunk)):
            for index, (ident, client) in reversed(list(enumerate(filters))):
                if mask & (1 << index):
                    continue
                if ident == 1:
                    raw = zlib.decompress(raw)
                elif ident == 2:
                    width = dtype.itemsize
                    raw = np.frombuffer(raw, dtype=np.uint8).reshape(width, -1).T.tobytes()
                else:
                    raise NotImplementedError(f"filter {ident}")
            block = np.frombuffer(raw[: int(np.prod(chunk)) * dtype.itemsize], dtype=dtype).reshape(chunk)
            where = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offsets, chunk, shape, strict=True))
            out[where] = block[tuple(slice(0, w.stop - w.start) for w in where)]
        return out.tobytes()

    def _chunks(self, address, rank):
        if self.data[address : address + 4] != b"TREE":
            raise ValueError("version 1 B-tree signature")
        level = self.data[address + 5]
        entries = self._u(address + 6, 2)
        p = address + 8 + 16  # left and right siblings
        key = 4 + 4 + 8 * (rank + 1)
        for _ in range(entries):
            size, mask = self._u(p, 4), self._u(p + 4, 4)
            offsets = tuple(self._u(p + 8 + 8 * d, 8) for d in range(rank))
            child = self._address(p + key)
            if level == 0:
                yield offsets, self.data[child : child + size], mask
            else:
                yield from self._chunks(child, rank)
            p += key + 8


class FractalHeap:
    """Managed objects of a fractal heap (specification section III.G): heap IDs resolve
    to the direct block that holds the object."""

    def __init__(self, f: HDF5File, address: int):
        d = f.data
        if d[address : address + 4] != b"FRHP":
            raise ValueError("fractal heap header signature")
        self.f = f
        self.id_length = f._u(address + 5, 2)
        filters_length = f._u(address + 7, 2)
        self.flags = d[address + 9]
        self.max_object = f._u(address + 10, 4)
        p = address + 14 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8
        self.width = f._u(p, 2)
        self.start_block = f._u(p + 2, 8)
        self.max_direct = f._u(p + 10, 8)
        self.max_heap_bits = f._u(p + 18, 2)
        self.root = f._address(p + 22)
        self.root_rows = f._u(p + 30, 2)
        if filters_length:
            raise NotImplementedError("filtered fractal heaps")
        self.offset_bytes = (self.max_heap_bits + 7) // 8
        self.length_bytes = (min(self.max_direct, self.max_object).bit_length() + 7) // 8
        self.blocks = []  # (heap offset, address, size) of every direct block
        if self.root_rows == 0:
            self.blocks.append((0, self.root, self.start_block))
        else:
            self._indirect(self.root, 0, self.root_rows)

    def _row_size(self, row: int) -> int:
        return self.start_block * (1 if row < 2 else 1 << (row - 1))

    def _indirect(self, address: int, heap_offset: int, rows: int):
        f = self.f
        if f.data[address : address + 4] != b"FHIB":
            raise ValueError("fractal heap indirect block signature")
        p = address + 5 + 8 + self.offset_bytes
        offset = heap_offset
        for row in range(rows):
            size = self._row_size(row)
            for _ in range(self.width):
                child = f._address(p)
                p += 8
                if size <= self.max_direct:
                    if child != UNDEFINED:
                        self.blocks.append((offset, child, size))
                else:
                    child_rows = (size // self.start_block).bit_length() - int.bit_length(self.width) + 1
                    if child != UNDEFINED:
                        self._indirect(child, offset, max(child_rows, 1))
                offset += size

    def locate(self, heap_id: bytes) -> int:
        """File offset of the managed object a heap ID names."""

        kind = (heap_id[0] >> 4) & 0x03
        if kind != 0:
            raise NotImplementedError("huge or tiny fractal heap objects")
        offset = int.from_bytes(heap_id[1 : 1 + self.offset_bytes], "little")
        for start, address, size in self.blocks:
            if start <= offset < start + size:
                if self.f.data[address : address + 4] != b"FHDB":
                    raise ValueError("fractal heap direct block signature")
                return address + (offset - start)
        raise ValueError(f"heap offset {offset} lies in no direct block")
