"""Reader/writer for the reference's JBinaryData container (``*.bi4`` files).

The layout follows the structure the reference documents and writes in
JBinaryData.h:461-489 and JBinaryData.cpp:736-1420 (``InItemBase``,
``InArrayBase``, ``SaveValues``, ``MakeFileHead``):

* a 64-byte head: ``"#FileJBD <code>"`` padded with spaces to 58 chars, ``\\n``,
  a zero, then byte-order (0 little-endian, +10 with 64-bit sizes) and si64;
* one item: ``uint sizedef`` then ``"\\nITEM\\n"``, name, hide, hidevalues,
  fmtfloat, fmtdouble, narrays, nitems, sizevalues; the values block
  (``"\\nVALUES"``, count, then name/type/value each); the arrays
  (``uint sizedef``, ``"\\nARRAY"``, name, hide, type, count, datasize, data);
  then the sub-items, recursively.

Strings are ``uint length`` + bytes, bools are 4-byte ints.  This is the format
``Case.bi4`` and ``data/Part_XXXX.bi4`` use (JPartDataBi4.cpp:169-470).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from typing import Any

import numpy as np

# JBinaryData.h:83-87 (TpData)
DAT_TEXT, DAT_BOOL, DAT_CHAR, DAT_UCHAR, DAT_SHORT, DAT_USHORT = 1, 2, 3, 4, 5, 6
DAT_INT, DAT_UINT, DAT_LLONG, DAT_ULLONG, DAT_FLOAT, DAT_DOUBLE = 7, 8, 9, 10, 11, 12
DAT_INT3, DAT_UINT3, DAT_FLOAT3, DAT_DOUBLE3 = 20, 21, 22, 23

_NP = {
    DAT_BOOL: (np.int32, 1), DAT_CHAR: (np.int8, 1), DAT_UCHAR: (np.uint8, 1),
    DAT_SHORT: (np.int16, 1), DAT_USHORT: (np.uint16, 1), DAT_INT: (np.int32, 1),
    DAT_UINT: (np.uint32, 1), DAT_LLONG: (np.int64, 1), DAT_ULLONG: (np.uint64, 1),
    DAT_FLOAT: (np.float32, 1), DAT_DOUBLE: (np.float64, 1), DAT_INT3: (np.int32, 3),
    DAT_UINT3: (np.uint32, 3), DAT_FLOAT3: (np.float32, 3), DAT_DOUBLE3: (np.float64, 3),
}
_SCALAR_FMT = {
    DAT_BOOL: "<i", DAT_CHAR: "<b", DAT_UCHAR: "<B", DAT_SHORT: "<h", DAT_USHORT: "<H",
    DAT_INT: "<i", DAT_UINT: "<I", DAT_LLONG: "<q", DAT_ULLONG: "<Q", DAT_FLOAT: "<f",
    DAT_DOUBLE: "<d", DAT_INT3: "<3i", DAT_UINT3: "<3I", DAT_FLOAT3: "<3f", DAT_DOUBLE3: "<3d",
}
CODE_ITEM = "\nITEM\n"
CODE_VALUES = "\nVALUES"
CODE_ARRAY = "\nARRAY"


class Bi4Error(ValueError):
    """Raised for malformed or unsupported bi4 content."""


@dataclass
class Item:
    """One JBinaryData item: ordered values, arrays and sub-items."""

    name: str
    values: dict[str, tuple[int, Any]] = field(default_factory=dict)
    arrays: dict[str, tuple[int, np.ndarray]] = field(default_factory=dict)
    items: list["Item"] = field(default_factory=list)
    hide: bool = False
    hidevalues: bool = False
    fmtfloat: str = "%.7E"
    fmtdouble: str = "%.15E"

    # -- values --
    def set(self, name: str, dtype: int, value: Any) -> None:
        self.values[name] = (dtype, value)

    def get(self, name: str, default: Any = None) -> Any:
        if name in self.values:
            return self.values[name][1]
        if default is not None:
            return default
        raise Bi4Error(f"value '{name}' not found in item '{self.name}'")

    def has(self, name: str) -> bool:
        return name in self.values

    # -- arrays --
    def set_array(self, name: str, dtype: int, data: np.ndarray) -> None:
        npt, width = _NP[dtype]
        arr = np.ascontiguousarray(np.asarray(data, dtype=npt))
        if width > 1:
            arr = arr.reshape(-1, width)
        self.arrays[name] = (dtype, arr)

    def array(self, name: str) -> np.ndarray:
        if name not in self.arrays:
            raise Bi4Error(f"array '{name}' not found in item '{self.name}'")
        return self.arrays[name][1]

    def item(self, name: str) -> "Item | None":
        for it in self.items:
            if it.name == name:
                return it
        return None


def _pstr(s: str) -> bytes:
    b = s.encode("latin-1")
    return struct.pack("<I", len(b)) + b


def _value_bytes(name: str, dtype: int, v: Any) -> bytes:
    out = _pstr(name) + struct.pack("<i", dtype)
    if dtype == DAT_TEXT:
        return out + _pstr(str(v))
    fmt = _SCALAR_FMT[dtype]
    if dtype in (DAT_INT3, DAT_UINT3, DAT_FLOAT3, DAT_DOUBLE3):
        return out + struct.pack(fmt, *v)
    if dtype == DAT_BOOL:
        return out + struct.pack(fmt, 1 if v else 0)
    return out + struct.pack(fmt, v)


def _values_block(item: Item) -> bytes:
    body = _pstr(CODE_VALUES) + struct.pack("<I", len(item.values))
    for k, (t, v) in item.values.items():
        body += _value_bytes(k, t, v)
    return body


def _item_bytes(item: Item, si64: bool) -> bytes:
    values = _values_block(item)
    base = (_pstr(CODE_ITEM) + _pstr(item.name) + struct.pack("<ii", int(item.hide), int(item.hidevalues))
            + _pstr(item.fmtfloat) + _pstr(item.fmtdouble)
            + struct.pack("<III", len(item.arrays), len(item.items), len(values)))
    out = [struct.pack("<I", len(base)), base, values]
    for name, (dtype, arr) in item.arrays.items():
        data = arr.tobytes()
        count = arr.shape[0] if arr.ndim else 1
        ab = _pstr(CODE_ARRAY) + _pstr(name) + struct.pack("<ii", 0, dtype)
        ab += struct.pack("<QQ", count, len(data)) if si64 else struct.pack("<II", count, len(data))
        out += [struct.pack("<I", len(ab)), ab, data]
    for sub in item.items:
        out.append(_item_bytes(sub, si64))
    return b"".join(out)


def write(path: str, root: Item) -> None:
    """Writes ``root`` as a JBinaryData file whose file code is ``root.name``."""
    body = _item_bytes(root, False)
    si64 = len(body) >= 4228102018  # JBinaryData::MaxSizeSi32
    if si64:
        body = _item_bytes(root, True)
    titu = ("#FileJBD " + root.name)[:58].ljust(58).encode("latin-1") + b"\n\x00"
    head = titu + bytes([10 if si64 else 0, 1 if si64 else 0, 0, 0])
    with open(path, "wb") as f:
        f.write(head)
        f.write(body)


class _Reader:
    def __init__(self, buf: bytes, si64: bool):
        self.b = memoryview(buf)
        self.o = 0
        self.si64 = si64

    def take(self, n: int) -> memoryview:
        if self.o + n > len(self.b):
            raise Bi4Error("overflow in reading data")
        v = self.b[self.o:self.o + n]
        self.o += n
        return v

    def u32(self) -> int:
        return struct.unpack("<I", self.take(4))[0]

    def i32(self) -> int:
        return struct.unpack("<i", self.take(4))[0]

    def size(self) -> int:
        return struct.unpack("<Q", self.take(8))[0] if self.si64 else self.u32()

    def pstr(self) -> str:
        n = self.u32()
        return bytes(self.take(n)).decode("latin-1")

    def value(self, item: Item) -> None:
        name = self.pstr()
        dtype = self.i32()
        if dtype == DAT_TEXT:
            item.values[name] = (dtype, self.pstr())
            return
        fmt = _SCALAR_FMT.get(dtype)
        if fmt is None:
            raise Bi4Error(f"invalid value type {dtype}")
        vals = struct.unpack(fmt, self.take(struct.calcsize(fmt)))
        v: Any = vals if len(vals) > 1 else vals[0]
        if dtype == DAT_BOOL:
            v = bool(v)
        item.values[name] = (dtype, v)

    def item(self) -> Item:
        _ = self.u32()  # size of the item definition
        if self.pstr() != CODE_ITEM:
            raise Bi4Error("validation code is invalid (ITEM)")
        it = Item(self.pstr())
        it.hide = bool(self.i32())
        it.hidevalues = bool(self.i32())
        it.fmtfloat = self.pstr()
        it.fmtdouble = self.pstr()
        narrays, nitems, sizevalues = self.u32(), self.u32(), self.u32()
        if sizevalues:
            if self.pstr() != CODE_VALUES:
                raise Bi4Error("validation code is invalid (VALUES)")
            for _ in range(self.u32()):
                self.value(it)
        for _ in range(narrays):
            _ = self.u32()
            if self.pstr() != CODE_ARRAY:
                raise Bi4Error("validation code is invalid (ARRAY)")
            name = self.pstr()
            _hide = self.i32()
            dtype = self.i32()
            count = self.size()
            sdata = self.size()
            if dtype == DAT_TEXT:
                it.arrays[name] = (dtype, np.array([self.pstr() for _ in range(count)], dtype=object))
                continue
            npt, width = _NP[dtype]
            if sdata != np.dtype(npt).itemsize * width * count:
                raise Bi4Error(f"size of data is invalid for array '{name}'")
            arr = np.frombuffer(bytes(self.take(sdata)), dtype=npt).copy()
            if width > 1:
                arr = arr.reshape(-1, width)
            it.arrays[name] = (dtype, arr)
        for _ in range(nitems):
            it.items.append(self.item())
        return it


def read(path: str, filecode: str | None = None) -> Item:
    """Reads a JBinaryData file and returns its root item."""
    with open(path, "rb") as f:
        raw = f.read()
    if len(raw) < 64:
        raise Bi4Error(f"file too small to be a JBinaryData file: {path}")
    head = raw[:64]
    titu = head[:60].decode("latin-1")
    if not titu.startswith("#FileJBD"):
        raise Bi4Error(f"the format file JBinaryData is invalid: {path}")
    if filecode is not None and titu[9:9 + len(filecode)] != filecode:
        raise Bi4Error(f"the file code is invalid: {path}")
    si64 = head[61] != 0
    byteorder = head[60] - (10 if si64 else 0)
    if byteorder != 0:
        raise Bi4Error(f"the byte-order in file is invalid: {path}")
    r = _Reader(raw[64:], si64)
    return r.item()


# ---------------------------------------------------------------------------
# JPartDataBi4 helpers (JPartDataBi4.cpp:169-470).
# ---------------------------------------------------------------------------
def make_partdata_root(*, casename: str, appname: str, data2d: bool, casenp: int, casenfixed: int,
                       casenmoving: int, casenfloat: int, casenfluid: int, caseposmin, caseposmax,
                       dp: float, h: float, b: float, rhop0: float, gamma: float, massbound: float,
                       massfluid: float, mapposmin=(0.0, 0.0, 0.0), mapposmax=(0.0, 0.0, 0.0)) -> Item:
    """Root item with the values JPartDataBi4::Config* writes."""
    d = Item("JPartDataBi4")
    d.set("Piece", DAT_UINT, 0)
    d.set("Npiece", DAT_UINT, 1)
    d.set("RunCode", DAT_TEXT, "00000000")
    d.set("Date", DAT_TEXT, "???")
    d.set("AppName", DAT_TEXT, appname)
    d.set("CaseName", DAT_TEXT, casename)
    d.set("Data2d", DAT_BOOL, data2d)
    d.set("Data2dPosY", DAT_DOUBLE, 0.0)
    d.set("MapPosMin", DAT_DOUBLE3, tuple(float(v) for v in mapposmin))
    d.set("MapPosMax", DAT_DOUBLE3, tuple(float(v) for v in mapposmax))
    d.set("PeriMode", DAT_INT, 0)
    d.set("PeriXinc", DAT_DOUBLE3, (0.0, 0.0, 0.0))
    d.set("PeriYinc", DAT_DOUBLE3, (0.0, 0.0, 0.0))
    d.set("PeriZinc", DAT_DOUBLE3, (0.0, 0.0, 0.0))
    d.set("AxisDiv", DAT_INT, 0)
    d.set("CaseNp", DAT_ULLONG, casenp)
    d.set("CaseNfixed", DAT_ULLONG, casenfixed)
    d.set("CaseNmoving", DAT_ULLONG, casenmoving)
    d.set("CaseNfloat", DAT_ULLONG, casenfloat)
    d.set("CaseNfluid", DAT_ULLONG, casenfluid)
    d.set("CasePosMin", DAT_DOUBLE3, tuple(float(v) for v in caseposmin))
    d.set("CasePosMax", DAT_DOUBLE3, tuple(float(v) for v in caseposmax))
    d.set("NpDynamic", DAT_BOOL, False)
    d.set("ReuseIds", DAT_BOOL, False)
    d.set("Dp", DAT_DOUBLE, dp)
    d.set("H", DAT_DOUBLE, h)
    d.set("B", DAT_DOUBLE, b)
    d.set("Rhop0", DAT_DOUBLE, rhop0)
    d.set("Gamma", DAT_DOUBLE, gamma)
    d.set("MassBound", DAT_DOUBLE, massbound)
    d.set("MassFluid", DAT_DOUBLE, massfluid)
    d.set("Symmetry", DAT_BOOL, False)
    d.set("Splitting", DAT_BOOL, False)
    return d


def make_part(cpart: int, timestep: float, npok: int, nout: int, step: int, domainmin, domainmax,
              idp, pos, vel, rhop, posdouble: bool, boundnor=None, extra: dict | None = None) -> Item:
    """Item ``PART_%04u`` with the values and arrays JPartDataBi4::AddPartInfo/AddPartData write."""
    p = Item("PART_%04u" % cpart)
    p.set("Cpart", DAT_UINT, cpart)
    p.set("TimeStep", DAT_DOUBLE, float(timestep))
    p.set("Npok", DAT_UINT, int(npok))
    p.set("Nout", DAT_UINT, int(nout))
    p.set("Step", DAT_UINT, int(step))
    p.set("RunTime", DAT_DOUBLE, 0.0)
    p.set("DomainMin", DAT_DOUBLE3, tuple(float(v) for v in domainmin))
    p.set("DomainMax", DAT_DOUBLE3, tuple(float(v) for v in domainmax))
    for k, (t, v) in (extra or {}).items():
        p.set(k, t, v)
    p.set_array("Idp", DAT_UINT, idp)
    if posdouble:
        p.set_array("Posd", DAT_DOUBLE3, pos)
    else:
        p.set_array("Pos", DAT_FLOAT3, np.asarray(pos, dtype=np.float32))
    p.set_array("Vel", DAT_FLOAT3, vel)
    p.set_array("Rhop", DAT_FLOAT, rhop)
    if boundnor is not None:
        p.set_array("BoundNor", DAT_FLOAT3, boundnor)
    return p
