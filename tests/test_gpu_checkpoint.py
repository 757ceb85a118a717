"""The device field registry and io::Checkpoint (src/io/Checkpoint.cpp:66-227)
on the GPU: the reference's checkpoint file (tests/golden/checkpoint_4x3x2,
written by the reference's own Checkpoint::write) is read into device memory
field for field and written back byte for byte (but for the timestamp); a
device SIMPLE run checkpointed and resumed continues exactly as an
uninterrupted one; damaged files are refused with a status."""
import os

import numpy as np
import pytest

from helpers import bits_equal

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURE = os.path.join(GOLD, "checkpoint_4x3x2.simallcp")

MESH_KEYS = {"node_x": "nx", "node_y": "ny", "node_z": "nz", "owner": "owner", "neighbor": "neighbor",
             "area_x": "ax", "area_y": "ay", "area_z": "az", "centroid_x": "fcx", "centroid_y": "fcy",
             "centroid_z": "fcz", "boundary_zone": "zone", "face_node_offsets": "fnOff",
             "face_node_indices": "fnIdx", "volume": "vol", "cell_centroid_x": "ccx", "cell_centroid_y": "ccy",
             "cell_centroid_z": "ccz", "cell_face_offsets": "cfOff", "cell_face_indices": "cfIdx"}


def _oracle_mesh_dict(om):
    d = {k: getattr(om, v) for k, v in MESH_KEYS.items()}
    for k in ("owner", "neighbor", "face_node_indices", "cell_face_indices"):
        d[k] = np.asarray(d[k]).astype(np.int64).view(np.uint64)
    return d


def test_reads_the_reference_checkpoint_and_writes_it_back(sg, ctx, tmp_path):
    g = np.load(os.path.join(GOLD, "checkpoint_4x3x2.npz"))
    reg = sg.DeviceFieldRegistry(ctx)
    meta, mesh = sg.checkpoint_read(FIXTURE, reg)
    assert meta == (17, 0.125, 0x123456789ABCDEF0)
    assert reg.names() == (["p", "T"], ["U"]) or sorted(reg.names()[0]) == ["T", "p"]
    assert bits_equal(reg.download("p"), g["p"]) and bits_equal(reg.download("T"), g["T"])
    assert bits_equal(reg.download("U", vector=True), g["U"])
    for k, v in MESH_KEYS.items():
        want = g[v]
        got = mesh[k]
        assert np.array_equal(got.view(np.uint8), np.ascontiguousarray(want).astype(got.dtype).view(np.uint8)), k
    out = str(tmp_path / "again.simallcp")
    sg.checkpoint_write(out, mesh, reg, *meta)
    a, b = open(FIXTURE, "rb").read(), open(out, "rb").read()
    assert len(a) == len(b)
    assert a[:16] == b[:16] and a[24:] == b[24:]  # bytes 16-23 hold the write time
    assert not os.path.exists(out + ".tmp")
    reg.close()


def test_registry_semantics(sg, ctx):
    """scalar()/vector() create zeroed fields and re-create them zeroed on a
    size change; find() reports absence."""
    reg = sg.DeviceFieldRegistry(ctx)
    assert reg.find("p") == (None, -1)
    reg.scalar("p", 5)
    assert np.array_equal(reg.download("p"), np.zeros(5))
    reg.upload("p", np.arange(5.0))
    reg.scalar("p", 5)  # same size: kept
    assert np.array_equal(reg.download("p"), np.arange(5.0))
    reg.scalar("p", 7)  # new size: zeroed
    assert np.array_equal(reg.download("p"), np.zeros(7))
    reg.vector("U", 4)
    assert reg.download("U", vector=True).shape == (3, 4) and reg.find("U", vector=True)[1] == 4
    assert reg.find("U")[1] == -1  # not a scalar
    reg.close()


def test_simple_resumes_from_a_checkpoint(sg, ctx, oracle, tmp_path):
    """Three outer iterations, checkpoint, a fresh algorithm reads it and runs
    two more: the same U and p as five uninterrupted iterations."""
    N = 16
    bcs = [(z, 1) for z in (1, 2, 3, 5, 6)] + [(4, 2, (1.0, 0.0, 0.0))]
    m = sg.cartesian(N, N, 1, 1.0, 1.0, 1.0 / N)
    om = oracle.cartesian_mesh(N, N, 1, 1.0, 1.0, 1.0 / N)

    def make(reg):
        mom = sg.make_linear_solver(sg.LinearSolverConfig(sg.LinearSolverKind.GMRES, sg.PreconditionerKind.ILU, 1e-8,
                                                          200, 30), ctx=ctx)
        pres = sg.GpuCGSolver(sg.LinearSolverConfig(sg.LinearSolverKind.CG, sg.PreconditionerKind.Jacobi, 1e-10,
                                                    2000), ctx=ctx)
        alg = sg.GpuSimpleAlgorithm(m, bcs, mom, pres, sg.SimpleOptions(mu=0.01), ctx=ctx)
        alg.bind_fields(reg)
        return alg, mom, pres

    r1 = sg.DeviceFieldRegistry(ctx)
    a1, m1, p1 = make(r1)
    for _ in range(5):
        a1.iterate()
    U5, p5, _ = a1.fields()
    r2 = sg.DeviceFieldRegistry(ctx)
    a2, m2, p2 = make(r2)
    for _ in range(3):
        a2.iterate()
    path = str(tmp_path / "simple.simallcp")
    sg.checkpoint_write(path, _oracle_mesh_dict(om), r2, iteration=3)
    r3 = sg.DeviceFieldRegistry(ctx)
    meta, _ = sg.checkpoint_read(path, r3, with_mesh=False)
    assert meta[0] == 3
    a3, m3, p3 = make(r3)
    for _ in range(2):
        a3.iterate()
    U, p, _ = a3.fields()
    assert bits_equal(U, U5) and bits_equal(p, p5)
    assert bits_equal(r3.download("U", vector=True), U5)
    for o in (a1, a2, a3, m1, m2, m3, p1, p2, p3, r1, r2, r3):
        o.close()


def test_damaged_files_are_refused(sg, ctx, tmp_path):
    reg = sg.DeviceFieldRegistry(ctx)
    with pytest.raises(sg.SimallError) as e:
        sg.checkpoint_read(str(tmp_path / "absent.simallcp"), reg)
    assert e.value.status == 14
    data = open(FIXTURE, "rb").read()
    bad = tmp_path / "bad.simallcp"
    bad.write_bytes(b"NOTSIMAL" + data[8:])
    with pytest.raises(sg.SimallError) as e:
        sg.checkpoint_read(str(bad), reg)
    assert e.value.status == 15
    newer = tmp_path / "newer.simallcp"
    newer.write_bytes(data[:8] + (2).to_bytes(4, "little") + data[12:])
    with pytest.raises(sg.SimallError) as e:
        sg.checkpoint_read(str(newer), reg)
    assert e.value.status == 15
    for cut in (20, 40, 200, len(data) - 5):
        short = tmp_path / f"short{cut}.simallcp"
        short.write_bytes(data[:cut])
        with pytest.raises(sg.SimallError) as e:
            sg.checkpoint_read(str(short), reg)
        assert e.value.status == 15, cut
    reg.close()


def test_reference_reads_our_checkpoint(sg, ctx, ref, tmp_path):
    """Where the compiled reference exists: its Checkpoint::read accepts a file
    written from device memory and finds every field."""
    g = np.load(os.path.join(GOLD, "checkpoint_4x3x2.npz"))
    reg = sg.DeviceFieldRegistry(ctx)
    _, mesh = sg.checkpoint_read(FIXTURE, reg)
    reg.upload("extra", np.linspace(0, 1, 24))
    out = str(tmp_path / "ours.simallcp")
    sg.checkpoint_write(out, mesh, reg, 5, 2.5, 99)
    md, meta, field = ref.checkpoint_read(out)
    assert meta == (5, 2.5, 99) and md["nC"] == 24
    assert bits_equal(field("p"), g["p"]) and bits_equal(field("U", True), g["U"])
    assert bits_equal(field("extra"), np.linspace(0, 1, 24))
    ref.free_mesh(md)
    reg.close()
