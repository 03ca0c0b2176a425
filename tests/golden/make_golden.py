"""Generate the committed golden fixtures from the channelflow reference's own test data.

Run where a channelflow checkout exists; its path is the first argument or,
failing that, the CHANNELFLOW_SRC environment variable:

    python tests/golden/make_golden.py /path/to/channelflow

It writes, next to this script:

* ``timeintegration.npz`` -- ``tests/data/uinit.nc`` and ``ufinal.nc`` of the
  reference's golden regression (``tests/timeIntegrationTest.cpp``): the
  physical velocity on the 32x35x32 I/O grid plus the file attributes.
* ``orrsommerfeld.npz`` -- the Orr-Sommerfeld eigenfunction data
  ``tests/data/os_ueig10_65.asc``, ``os_peig10_65.asc`` and the eigenvalue
  ``os_omega10_65.cmplx`` used by ``tests/dnsOrrsommTest.cpp``.

The netCDF-4 files are HDF5 containers; no HDF5 library is available here,
so this script carries a minimal reader for what those files use:
superblock v2, version-2 object headers with continuation chunks, compact
link messages, contiguous datasets of little-endian IEEE doubles, and
compact attributes.
"""

from __future__ import annotations

import os
import struct
import sys

import numpy as np


class H5Min:
    def __init__(self, path):
        self.d = open(path, "rb").read()
        d = self.d
        assert d[:8] == b"\x89HDF\r\n\x1a\n", "not an HDF5 file"
        ver = d[8]
        assert ver in (2, 3), "only superblock v2/v3 supported"
        so, sl = d[9], d[10]
        assert so == 8 and sl == 8
        self.root = struct.unpack_from("<Q", d, 12 + 8 * 3)[0]

    # -- object headers -------------------------------------------------
    def messages(self, addr):
        d = self.d
        out = []
        assert d[addr:addr + 4] == b"OHDR", "expected v2 object header at %d" % addr
        flags = d[addr + 5]
        p = addr + 6
        if flags & 0x20:
            p += 16
        if flags & 0x10:
            p += 4
        nsz = 1 << (flags & 3)
        chunk = int.from_bytes(d[p:p + nsz], "little")
        p += nsz
        blocks = [(p, p + chunk)]
        while blocks:
            start, end = blocks.pop(0)
            q = start
            while q + 4 <= end:
                mtype = d[q]
                msize = struct.unpack_from("<H", d, q + 1)[0]
                mflags = d[q + 3]
                q += 4
                if flags & 0x04:
                    q += 2
                body = d[q:q + msize]
                q += msize
                if mtype == 0x10:  # continuation
                    caddr, clen = struct.unpack_from("<QQ", body, 0)
                    assert d[caddr:caddr + 4] == b"OCHK"
                    blocks.append((caddr + 4, caddr + clen - 4))
                elif mtype != 0:
                    out.append((mtype, body))
        return out

    # -- decoders ---------------------------------------------------------
    @staticmethod
    def link(body):
        ver, fl = body[0], body[1]
        p = 2
        ltype = 0
        if fl & 0x08:
            ltype = body[p]
            p += 1
        if fl & 0x04:
            p += 8
        if fl & 0x10:
            p += 1
        nl = 1 << (fl & 3)
        ln = int.from_bytes(body[p:p + nl], "little")
        p += nl
        name = body[p:p + ln].decode()
        p += ln
        assert ltype == 0, "only hard links"
        addr = struct.unpack_from("<Q", body, p)[0]
        return name, addr

    @staticmethod
    def dataspace(body):
        ver = body[0]
        nd = body[1]
        if ver == 1:
            p = 8
        else:
            p = 4
        return tuple(struct.unpack_from("<%dQ" % nd, body, p)) if nd else ()

    @staticmethod
    def datatype(body):
        cls = body[0] & 0x0F
        size = struct.unpack_from("<I", body, 4)[0]
        bits0 = body[1]
        return cls, size, bits0

    def attributes(self, msgs):
        out = {}
        for t, b in msgs:
            if t != 0x0C:
                continue
            ver = b[0]
            nsz, tsz, ssz = struct.unpack_from("<HHH", b, 2)
            p = 8 if ver == 1 else (8 if ver == 2 else 9)
            name = b[p:p + nsz].split(b"\0")[0].decode()
            p += nsz if ver != 1 else (nsz + 7) // 8 * 8
            dt = b[p:p + tsz]
            p += tsz if ver != 1 else (tsz + 7) // 8 * 8
            ds = b[p:p + ssz]
            p += ssz if ver != 1 else (ssz + 7) // 8 * 8
            cls, size, _ = self.datatype(dt)
            shape = self.dataspace(ds)
            n = int(np.prod(shape)) if shape else 1
            raw = b[p:p + n * size]
            if cls == 1 and size == 8:
                v = np.frombuffer(raw, "<f8")
            elif cls == 0 and size == 4:
                v = np.frombuffer(raw, "<i4")
            elif cls == 0 and size == 8:
                v = np.frombuffer(raw, "<i8")
            else:
                v = raw
            out[name] = v[0] if hasattr(v, "shape") and v.shape == (1,) else v
        return out

    def dataset(self, addr):
        msgs = self.messages(addr)
        shape, dtype, layout = None, None, None
        for t, b in msgs:
            if t == 0x01:
                shape = self.dataspace(b)
            elif t == 0x03:
                dtype = self.datatype(b)
            elif t == 0x08:
                ver, cls = b[0], b[1]
                assert ver == 3
                if cls == 1:
                    layout = ("contiguous",) + struct.unpack_from("<QQ", b, 2)
                elif cls == 0:
                    sz = struct.unpack_from("<H", b, 2)[0]
                    layout = ("compact", b[4:4 + sz])
                else:
                    raise NotImplementedError("chunked layout")
            elif t == 0x0B:
                raise NotImplementedError("filtered dataset")
        cls, size, bits0 = dtype
        assert cls == 1 and size == 8 and not (bits0 & 1), "expected little-endian float64"
        n = int(np.prod(shape))
        if layout[0] == "contiguous":
            off = layout[1]
            raw = self.d[off:off + n * 8]
        else:
            raw = layout[1]
        return np.frombuffer(raw, "<f8").reshape(shape).copy()

    def dense_attributes(self, names):
        """Attributes kept in a fractal heap (Attribute Info message).

        Each heap object is a version-3 attribute message; rather than walk
        the heap's B-tree, locate each wanted name and decode the message that
        begins 9 bytes before it, checking the header fields for consistency.
        """
        out = {}
        d = self.d
        for nm in names:
            key = nm.encode() + b"\0"
            pos = d.find(key)
            while pos >= 0:
                st = pos - 9
                if st >= 0 and d[st] == 3:
                    nsz, tsz, ssz = struct.unpack_from("<HHH", d, st + 2)
                    if nsz == len(key) and 0 < tsz < 64 and 0 < ssz < 64:
                        body = d[st:st + 9 + nsz + tsz + ssz + 64]
                        got = self.attributes([(0x0C, body)])
                        if nm in got:
                            out[nm] = got[nm]
                            break
                pos = d.find(key, pos + 1)
        return out

    def read_all(self):
        msgs = self.messages(self.root)
        attrs = self.attributes(msgs)
        if any(t == 0x15 for t, _ in msgs):
            attrs.update(self.dense_attributes(["Nx", "Ny", "Nz", "Lx", "Lz", "a", "b"]))
        data = {}
        for t, b in msgs:
            if t == 0x06:
                name, addr = self.link(b)
                data[name] = self.dataset(addr)
        return attrs, data


def read_nc(path):
    attrs, data = H5Min(path).read_all()
    return attrs, data


def read_asc_basis(path):
    """BasisFunc .asc: header '% Nd Ny kx kz Lx Lz a b state', then Ny rows of Nd (re, im) pairs."""
    with open(path) as f:
        head = f.readline().split()
        assert head[0] == "%"
        Nd, Ny = int(head[1]), int(head[2])
        vals = np.loadtxt(f).reshape(Ny, Nd, 2)
    return vals[..., 0] + 1j * vals[..., 1], head


def main(ref=None):
    ref = ref or os.environ.get("CHANNELFLOW_SRC")
    if not ref:
        raise SystemExit("usage: make_golden.py /path/to/channelflow (or set CHANNELFLOW_SRC)")
    here = os.path.dirname(os.path.abspath(__file__))
    dd = os.path.join(ref, "tests", "data")
    out = {}
    for tag in ("uinit", "ufinal"):
        attrs, data = read_nc(os.path.join(dd, tag + ".nc"))
        vel = np.stack([data["Velocity_X"], data["Velocity_Y"], data["Velocity_Z"]])
        out[tag] = vel
        for k in ("Nx", "Ny", "Nz", "Lx", "Lz", "a", "b"):
            out[tag + "_" + k] = np.asarray(attrs[k])
        for k in ("X", "Y", "Z"):
            out[tag + "_coord_" + k] = data[k]
    np.savez_compressed(os.path.join(here, "timeintegration.npz"), **out)
    # the equilibrium (travelling wave) of tests/findsolnTest.cpp and its symmetry (x shift) sigmabest.asc
    attrs, data = read_nc(os.path.join(dd, "eq.nc"))
    eq = {"eq": np.stack([data["Velocity_X"], data["Velocity_Y"], data["Velocity_Z"]])}
    for k in ("Nx", "Ny", "Nz", "Lx", "Lz", "a", "b"):
        eq["eq_" + k] = np.asarray(attrs[k])
    eq["sigmabest"] = np.loadtxt(os.path.join(dd, "sigmabest.asc"))
    np.savez_compressed(os.path.join(here, "eq.npz"), **eq)
    ueig, uhead = read_asc_basis(os.path.join(dd, "os_ueig10_65.asc"))
    peig, phead = read_asc_basis(os.path.join(dd, "os_peig10_65.asc"))
    om = np.loadtxt(os.path.join(dd, "os_omega10_65.cmplx"))
    np.savez_compressed(os.path.join(here, "orrsommerfeld.npz"), ueig=ueig, peig=peig,
                        omega=np.array(om[0] + 1j * om[1]), header=np.array(" ".join(uhead)))
    print("wrote fixtures to", here)


if __name__ == "__main__":
    main(*sys.argv[1:])
