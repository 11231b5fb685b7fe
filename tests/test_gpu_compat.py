"""libmat's C++ entry point, compute_clipped_voro_diagram_GPU (the header-only
shim include/rpd_gb300_compat.hpp over the C ABI), driven by a C++ program
with the reference's input layouts; its ConvexCellHost records must be the
reference's own cells (golden fixtures made by the reference's kernel code),
thread ids included."""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import ROOT
from tests.helpers import SUCCESS, float_vertices, ref_headers, section_sizes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def compat_exe(tmp_path_factory):
    from libmat_gb300 import build as libbuild

    lib = libbuild.build()
    out = str(tmp_path_factory.mktemp("compat") / "compat_main")
    cuda_inc = os.path.join(libbuild.cuda_home(), "include")
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", os.path.join(ROOT, "tests", "cpp", "compat_main.cpp"),
                    "-I" + os.path.join(ROOT, "include"), "-I" + cuda_inc, "-o", out,
                    lib, "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return out


def write_input(path, c):
    vert = c["vert3d"].astype(np.float32)
    tets = c["tets"].astype(np.int32)
    n_vert, n_tet, n_site = vert.shape[0], tets.shape[0], c["sites"].shape[0]
    nbr = c["nbr"]
    k = nbr.shape[1]
    site_knn = np.full((k + 1, n_site), -1, np.int32)
    site_knn[:k] = nbr.T
    e_adjs = O.dense_e_adjs(n_vert, tets, c["e_adj6"])
    s4 = c["sites"].astype(np.float32)
    with open(path, "wb") as f:
        np.array([n_vert, n_tet, n_site, k], np.int32).tofile(f)
        vert.tofile(f)
        tets.tofile(f)
        c["v_adjs"].astype(np.int32).tofile(f)
        np.array([e_adjs.size], np.int32).tofile(f)
        e_adjs.tofile(f)
        c["f_adjs"].astype(np.int32).tofile(f)
        c["f_ids"].astype(np.int32).tofile(f)
        np.ascontiguousarray(s4[:, :3].T).tofile(f)
        s4[:, 3].tofile(f)
        c["flags"].astype(np.uint32).tofile(f)
        site_knn.tofile(f)


def topo_sections(rec, th, nv, np_, ne):
    o = int(th["offset"])
    return (rec[o:o + 4 * np_].view(np.float32), rec[o + 4 * np_:o + 5 * np_],
            rec[o + 5 * np_:o + 6 * np_].view(np.int8), rec[o + 6 * np_:o + 6 * np_ + ne],
            rec[o + 6 * np_ + ne:o + 6 * np_ + ne + 3 * nv])


@pytest.mark.parametrize("name", ["random_full", "cube_k64", "dups_flags_holes", "lattice_ties"])
def test_compat_entry_point_returns_reference_cells(golden_cases, compat_exe, tmp_path, name):
    c = golden_cases[name]
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, c)
    subprocess.run([compat_exe, inp, outp], check=True)
    raw = np.fromfile(outp, np.uint8)
    rh = ref_headers(c)
    ok = np.flatnonzero(rh["status"] == SUCCESS)
    th_ref = c["topo_headers"].reshape(-1).view(O.TOPO_DTYPE)
    trec_ref = c["topo_records"]
    n = int(raw[:4].view(np.int32)[0])
    assert n == len(ok)
    pos = 4
    for j, q in enumerate(ok):
        h = raw[pos:pos + 32].view(np.int32)
        pos += 32
        status, tid, voro, tet, cid, nv, np_, ne = [int(x) for x in h]
        assert (status, voro, tet, cid) == (SUCCESS, int(rh["site_id"][q]), int(rh["tet_id"][q]), j)
        assert tid == int(c["ref_thread_ids"][q])
        assert (nv, np_, ne) == (int(rh["nb_v"][q]), int(rh["nb_p"][q]), int(rh["nb_e"][q]))
        s = section_sizes(nv, np_, ne)
        base = int(rh["offset"][q])
        ref = c["ref_payload"]
        ver = raw[pos:pos + 4 * nv]
        pos += 4 * nv
        assert np.array_equal(ver, ref[base + s["plane"] + s["id2"]:][:4 * nv])
        planes = raw[pos:pos + 20 * np_].view(np.float32).reshape(-1, 5)
        pos += 20 * np_
        assert np.array_equal(planes[:, :4], ref[base:base + 16 * np_].view(np.float32).reshape(-1, 4))
        assert np.array_equal(planes[:, 4], ref[base + s["plane"] + s["id2"] + s["ver"] + s["edge"]:][:np_].astype(np.float32))
        ids = raw[pos:pos + 8 * np_].view(np.int32)
        pos += 8 * np_
        assert np.array_equal(ids, ref[base + s["plane"]:][:8 * np_].view(np.int32))
        edges = raw[pos:pos + 3 * ne].reshape(-1, 3)
        pos += 3 * ne
        ref_e = ref[base + s["plane"] + s["id2"] + s["ver"]:][:4 * ne].reshape(-1, 4)[:, :3]
        assert np.array_equal(edges, ref_e)
        # topology filled by the shim = the reference's own reload_active /
        # reload_pc_explicit (golden topology of the same cell)
        upd, expl, nf = [int(x) for x in raw[pos:pos + 12].view(np.int32)]
        pos += 12
        assert upd == 1 and expl == 1
        gh = th_ref[j]
        facet, gact, glf, gacte, gfaces = topo_sections(trec_ref, gh, nv, np_, ne)
        assert nf == int(gh["n_faces"])
        act = raw[pos:pos + 4 * (np_ + 1)].view(np.int32)
        pos += 4 * (np_ + 1)
        assert np.array_equal(act[:np_], gact) and act[np_] == 0
        acte = raw[pos:pos + 4 * (ne + 1)].view(np.int32)
        pos += 4 * (ne + 1)
        assert np.array_equal(acte[:ne], gacte) and acte[ne] == 0
        faces = []
        for _ in range(nf):
            m = int(raw[pos:pos + 4].view(np.int32)[0])
            faces.extend(raw[pos + 4:pos + 4 + 4 * m].view(np.int32).tolist())
            pos += 4 + 4 * m
        assert faces == gfaces.tolist()
        lf = raw[pos:pos + 4 * np_].view(np.int32)
        pos += 4 * np_
        assert np.array_equal(lf, glf)
        pts = raw[pos:pos + 12 * nv].view(np.float32).reshape(-1, 3)
        pos += 12 * nv
        assert np.array_equal(pts, float_vertices(planes[:, :4], ver.reshape(-1, 4)))
    vol = raw[pos:].view(np.float32)
    assert vol.shape[0] == c["sites"].shape[0]
