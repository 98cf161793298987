"""Oracle (test infrastructure only): the .gt binary format of graph-tool-rs.

A plain-Python restatement of the reference's reader and writer,
crates/gt-io/src/gt.rs of graph-tool-rs:

  read            gt.rs:555-626   header, adjacency, property table
  read_adjacency  gt.rs:628-678   one (count, list) record per vertex; an
                                  entry u of v's list is add_edge(v, u), in
                                  file order, after the check u < N (:658-664)
  vint_width      gt.rs:689-699   index width 1/2/4/8 bytes by N
  read_column     gt.rs:724-820   one value per element of the domain
  write           gt.rs:865-903   magic, version, host byte order, comment,
                                  adjacency, properties grouped by domain
  write_adjacency gt.rs:905-940   out-edges of each vertex in edge-id order
  generated_comment gt.rs:361-373

The tests use it to check the library's reader (gtc_gt_open / gtc_gt_graph)
and to write documents of every value kind in either byte order.  It is
never part of the product path.
"""
from __future__ import annotations

import struct

MAGIC = "⛾ gt".encode()  # gt.rs:64
VERSION = 1                    # gt.rs:74

# ValueKind::ALL, crates/gt-core/src/prop/value.rs:79-95
KINDS = ["bool", "int16_t", "int32_t", "int64_t", "double", "long double", "string",
         "vector<bool>", "vector<int16_t>", "vector<int32_t>", "vector<int64_t>",
         "vector<double>", "vector<long double>", "vector<string>", "python::object"]
_SCALAR = {0: "B", 1: "h", 2: "i", 3: "q", 4: "d"}
_VEC_OF = {8: "h", 9: "i", 10: "q", 11: "d"}
GRAPH, VERTEX, EDGE = 0, 1, 2


class GtError(Exception):
    """IoError (crates/gt-io/src/error.rs): .kind names the variant."""

    def __init__(self, kind: str, msg: str):
        super().__init__(f"{kind}: {msg}")
        self.kind = kind


def vint_width(n: int) -> int:
    if n <= 0xFF:
        return 1
    if n <= 0xFFFF:
        return 2
    if n <= 0xFFFFFFFF:
        return 4
    return 8


class _Src:
    def __init__(self, b: bytes):
        self.b, self.pos, self.big = b, 0, False

    def exact(self, k: int) -> bytes:
        if k > len(self.b) - self.pos:
            raise GtError("Parse", f"at byte {self.pos}: unexpected end of file, wanted {k} more bytes")
        out = self.b[self.pos:self.pos + k]
        self.pos += k
        return out

    def num(self, fmt: str):
        size = struct.calcsize(fmt)
        return struct.unpack((">" if self.big else "<") + fmt, self.exact(size))[0]

    def u8(self) -> int:
        return self.exact(1)[0]

    def u64(self) -> int:
        return self.num("Q")

    def bytes_(self) -> bytes:
        n = self.u64()
        at = self.pos
        if n > len(self.b) - self.pos:
            raise GtError("Parse", f"at byte {at}: string declares {n} bytes, "
                                   f"{len(self.b) - self.pos} are present")
        out = self.b[self.pos:self.pos + n]
        self.pos += n
        return out

    def text(self, what: str) -> str:
        at = self.pos
        b = self.bytes_()
        try:
            return b.decode("utf-8")
        except UnicodeDecodeError as e:
            raise GtError("Parse", f"at byte {at}: {what} is not valid UTF-8 at offset {e.start}")

    def value_str(self, name: str, kind: int) -> str:
        b = self.bytes_()
        try:
            return b.decode("utf-8")
        except UnicodeDecodeError:
            raise GtError("MalformedProperty", f"{name} declared {KINDS[kind]}")


def read(b: bytes) -> dict:
    """gt.rs:555-626.  Returns n, directed, big_endian, comment, src, tgt
    (edge k = the k-th list entry in file order) and props, a list of
    (name, domain, kind, values)."""
    s = _Src(bytes(b))
    head = s.b[:6]
    if len(head) != 6 or head != MAGIC:
        raise GtError("BadMagic", f"found {head!r}")
    s.pos = 6
    version = s.u8()
    if version != VERSION:
        raise GtError("UnsupportedVersion", str(version))
    s.big = s.u8() != 0
    comment = s.text("the header comment")
    directed = s.u8() != 0
    n = s.u64()
    if n > 0 and n - 1 > 0xFFFFFFFE:
        raise GtError("IndexWidthExceeded", str(n))
    width = vint_width(n)
    fmt = {1: "B", 2: "H", 4: "I", 8: "Q"}[width]
    src, tgt = [], []
    for v in range(n):
        k = s.u64()
        for _ in range(k):
            u = s.num(fmt)
            if u >= n:
                raise GtError("IndexOutOfRange", f"vertex index {u} bound {n}")
            src.append(v)
            tgt.append(u)
    m = len(src)
    props = []
    for _ in range(s.u64()):
        at = s.pos
        dom = s.u8()
        if dom > 2:
            raise GtError("Parse", f"at byte {at}: invalid property domain {dom}")
        name = s.text("a property name")
        kind = s.u8()
        if kind >= len(KINDS):
            raise GtError("UnknownValueType", f"value type index {kind}")
        count = 1 if dom == GRAPH else (n if dom == VERTEX else m)
        props.append((name, dom, kind, _column(s, kind, count, name)))
    return dict(n=n, directed=directed, big_endian=s.big, comment=comment, src=src, tgt=tgt,
                props=props)


def _column(s: _Src, kind: int, count: int, name: str) -> list:
    """read_column, gt.rs:724-820."""
    out = []
    for _ in range(count):
        if kind in _SCALAR:
            out.append(s.num(_SCALAR[kind]))
        elif kind == 5:
            b = s.exact(16)
            out.append(b[::-1] if s.big else b)  # opaque, reversed into host order
        elif kind == 6:
            out.append(s.value_str(name, kind))
        elif kind in (7, 14):
            out.append(s.bytes_())
        elif kind in _VEC_OF:
            out.append([s.num(_VEC_OF[kind]) for _ in range(s.u64())])
        elif kind == 12:
            k = s.u64()
            out.append([s.exact(16) for _ in range(k)])
        else:  # 13: vector<string>
            k = s.u64()
            out.append([s.value_str(name, kind) for _ in range(k)])
    return out


def write(n: int, edges, directed: bool = True, props=(), comment: str | None = None,
          big_endian: bool = False) -> bytes:
    """write, gt.rs:865-903.  ``edges`` is the (src, tgt) list in edge-id
    order; ``props`` a list of (name, domain, kind, values), edge columns by
    edge id.  ``big_endian`` writes the document a big-endian host would."""
    e = "<>"[bool(big_endian)]
    out = bytearray(MAGIC)
    out.append(VERSION)
    out.append(1 if big_endian else 0)
    if comment is None:  # generated_comment, gt.rs:361-373
        ng = sum(1 for p in props if p[1] == GRAPH)
        nv = sum(1 for p in props if p[1] == VERTEX)
        ne = sum(1 for p in props if p[1] == EDGE)
        comment = (f"graph-tool binary file version {VERSION} (https://graph-tool.skewed.de), "
                   f"stats: {n} vertices, {len(edges)} edges, "
                   f"{'directed' if directed else 'undirected'}, {ng} graph props, "
                   f"{nv} vertex props, {ne} edge props")

    def put_bytes(b: bytes):
        out.extend(struct.pack(e + "Q", len(b)))
        out.extend(b)

    put_bytes(comment.encode())
    # write_adjacency, gt.rs:905-940: out-edges of each vertex in edge-id order
    out.append(1 if directed else 0)
    out.extend(struct.pack(e + "Q", n))
    fmt = {1: "B", 2: "H", 4: "I", 8: "Q"}[vint_width(n)]
    outl = [[] for _ in range(n)]
    for k, (s_, t_) in enumerate(edges):
        outl[s_].append((k, t_))
    order = []
    for v in range(n):
        out.extend(struct.pack(e + "Q", len(outl[v])))
        for k, t_ in outl[v]:
            out.extend(struct.pack(e + fmt, t_))
            order.append(k)
    out.extend(struct.pack(e + "Q", len(props)))
    for dom in (GRAPH, VERTEX, EDGE):  # grouped by domain, gt.rs:886-897
        for name, d, kind, values in props:
            if d != dom:
                continue
            out.append(d)
            put_bytes(name.encode())
            out.append(kind)
            idx = [0] if d == GRAPH else (range(n) if d == VERTEX else order)
            for i in idx:
                x = values[i]
                if kind in _SCALAR:
                    out.extend(struct.pack(e + _SCALAR[kind], x))
                elif kind == 5:
                    out.extend(x[::-1] if big_endian else x)
                elif kind == 6:
                    put_bytes(x.encode())
                elif kind in (7, 14):
                    put_bytes(bytes(x))
                elif kind in _VEC_OF:
                    out.extend(struct.pack(e + "Q", len(x)))
                    for y in x:
                        out.extend(struct.pack(e + _VEC_OF[kind], y))
                elif kind == 12:
                    out.extend(struct.pack(e + "Q", len(x)))
                    for y in x:
                        out.extend(y[::-1] if big_endian else y)
                else:
                    out.extend(struct.pack(e + "Q", len(x)))
                    for y in x:
                        put_bytes(y.encode())
    return bytes(out)
