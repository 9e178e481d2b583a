"""VTU output (cfdl_write_vtu) against a restatement of the reference's
write_vtubin (src/modules/mod_vtu_output.f90:6-328) in this test: the file
must be the same bytes, and its values the case's fields."""
import struct

import numpy as np
import pytest

import cfdl

pytestmark = pytest.mark.gpu

VTK = {10: 10, 17: 12, 12: 14, 14: 13}
NVX = {10: 4, 17: 8, 12: 5, 14: 6}


def i12(v):
    return "%12d" % v


def uvwp_vars(s, fields):
    """write_vtubin's variable list for the uvwp equation (mod_vtu_output.f90:101-123)."""
    ne = s.ne
    idx, ef2 = s.get_int("ef2nb_idx"), s.get_int("ef2nb2")
    mip = fields["mip"]
    net = np.zeros(ne)
    for e in range(ne):
        for h in range(idx[e], idx[e + 1]):
            fg = int(ef2[h - 1])
            sg = 1 if fg > 0 else -1
            net[e] = net[e] + mip[abs(fg) - 1] * sg
    return [("u", 1, fields["u"]), ("v", 1, fields["v"]), ("w", 1, fields["w"]), ("p", 1, fields["p"]),
            ("gpc", 3, fields["gpc"]), ("mip", 1, net)]


def restated_vtu(s, fields, vars_):
    """Bytes of write_vtubin for the variable list vars_ (test restatement)."""
    ne, nvx = s.ne, fields["nvx"]
    esec, etype = s.get_int("esec"), s.get_int("etype")
    vol = [(int(esec[2 * q]), int(esec[2 * q + 1]), int(etype[q])) for q in range(s.nsec) if etype[q] >= 10]
    lf = "\n"
    out = [b'<?xml version="1.0"?>' + b"\n",
           b'<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n',
           b" <UnstructuredGrid>\n",
           ('  <Piece NumberOfPoints="%d" NumberOfCells="%d">' % (nvx, ne) + lf).encode(),
           b'   <CellData Scalars="scalars">\n']
    off = 0
    for name, dim, _ in vars_:
        out.append(('    <DataArray type="Float64" Name="%s" NumberOfComponents="%d" format="appended" offset="%s" />'
                    % (name, dim, i12(off)) + lf).encode())
        off += 8 + ne * dim * 8
    nconn = sum((b - a + 1) * NVX[t] for a, b, t in vol)
    ncell = sum(b - a + 1 for a, b, t in vol)
    out.append(b"   </CellData>\n")
    out.append(b"   <Points>\n")
    out.append(('    <DataArray type="Float64" NumberOfComponents="3" format="appended" offset="%s" />' % i12(off) + lf).encode())
    off += 8 + 3 * nvx * 8
    out.append(b"   </Points>\n")
    out.append(b"   <Cells>\n")
    out.append(('    <DataArray type="Int32" Name="connectivity" format="appended" offset="%s" />' % i12(off) + lf).encode())
    off += 8 + nconn * 4
    out.append(('    <DataArray type="Int32" Name="offsets" format="appended" offset="%s" />' % i12(off) + lf).encode())
    off += 8 + ncell * 4
    out.append(('    <DataArray type="Int32" Name="types" format="appended" offset="%s" />' % i12(off) + lf).encode())
    out += [b"   </Cells>\n", b"  </Piece>\n", b" </UnstructuredGrid>\n", b' <AppendedData encoding="raw">\n', b"_"]
    for name, dim, a in vars_:
        out.append(struct.pack("<Q", ne * dim * 8))
        for a0, b0, t in vol:
            out.append(np.ascontiguousarray(a[(a0 - 1) * dim:b0 * dim], dtype="<f8").tobytes())
    out.append(struct.pack("<Q", 3 * nvx * 8))
    out.append(np.stack([fields["x"], fields["y"], fields["z"]], axis=1).astype("<f8").tobytes())
    e2vx, m = fields["e2vx"], fields["m"]
    out.append(struct.pack("<Q", nconn * 4))
    for a0, b0, t in vol:
        blk = e2vx.reshape(-1, m)[a0 - 1:b0, :NVX[t]] - 1
        out.append(blk.astype("<i4").tobytes())
    out.append(struct.pack("<Q", ncell * 4))
    l, offs = 0, []
    for a0, b0, t in vol:
        for _ in range(a0, b0 + 1):
            l += NVX[t]
            offs.append(l)
    out.append(np.array(offs, dtype="<i4").tobytes())
    out.append(struct.pack("<Q", ne * 4))
    for a0, b0, t in vol:
        out.append(np.full(b0 - a0 + 1, VTK[t], dtype="<i4").tobytes())
    out.append(b"\n </AppendedData>\n</VTKFile>\n")
    return b"".join(out)


@pytest.mark.parametrize("n,tet", [(5, False), (4, True), (3, "prism"), (3, "mixed")])
def test_vtu_bytes_match_the_reference_layout(need_gpu, tmp_path, n, tet):
    z = cfdl.Zone(n, tet, 0.1, seed=3)
    s = cfdl.Setup(z)
    g = cfdl.Solver(s, cfdl.steady())
    g.step(4, ncoef=0)
    path = tmp_path / "uvwp.vtu"
    g.write_vtu(path)
    fields = {f: g.get(f) for f in ("u", "v", "w", "p", "gpc", "mip")}
    fields.update(x=z.x, y=z.y, z=z.z, nvx=z.nvx, e2vx=z.e2vx, m=z.ne2vxmax)
    got = path.read_bytes()
    want = restated_vtu(s, fields, uvwp_vars(s, fields))
    assert got == want
    g.close()


def test_vtu_energy_bytes(need_gpu, tmp_path):
    """write_vtubin for the energy equation (mod_vtu_output.f90:124-132)."""
    z = cfdl.Zone(4, True, 0.1, seed=5)
    s = cfdl.Setup(z)
    g = cfdl.Solver(s, cfdl.default_config())
    with pytest.raises(cfdl.CfdlError):
        g.write_vtu_energy(tmp_path / "none.vtu")
    g.energy_init()
    g.step(3, ncoef=3)
    path = tmp_path / "energy.vtu"
    g.write_vtu_energy(path)
    f = {k: g.get(k) for k in ("e", "ge", "t", "gt")}
    vars_ = [("enthalpy", 1, f["e"]), ("grad_enthalpy", 3, f["ge"]), ("temperature", 1, f["t"]),
             ("grad_temperature", 3, f["gt"])]
    fields = dict(x=z.x, y=z.y, z=z.z, nvx=z.nvx, e2vx=z.e2vx, m=z.ne2vxmax)
    assert path.read_bytes() == restated_vtu(s, fields, vars_)
    g.close()
