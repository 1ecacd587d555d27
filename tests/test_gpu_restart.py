"""Restart particle section and particle checksum (pic_restart.cpp) against
the oracle: the device-packed section is byte-identical to the oracle's pack
of the same particles (block order, node ids, cell tables, records in reverse
list order), the device checksum equals the oracle's CRC32 walk, and a section
read back restores every cell's list, so that the checksum, the exported
particles and the next step are those of the saved state."""
import numpy as np
import pytest

import amps_gb300 as A
from amps_gb300._capi import AmpsGpuError, RecordLayout
from tests import gpu_cases as G
from tests import oracle_lib as O
from tests.test_gpu_amr import amr_case, gpu_for

pytestmark = pytest.mark.gpu

LAYOUTS = [RecordLayout.basic(False), RecordLayout.basic(True), RecordLayout(96, 24, 56, 88, -1)]


def _oracle_inputs(exp, wc_by_id=None):
    wc = None if wc_by_id is None else wc_by_id[exp["id"]]
    return exp["x"], exp["v"], exp["spec"], exp["block"], exp["cell"], wc


def _random_ids(nb, length, seed):
    rng = np.random.default_rng(seed)
    ids = rng.integers(0, 256, size=(nb, length), dtype=np.uint8)
    ids[:, 0] = np.arange(nb) % 256          # unique
    ids[:, 1] = np.arange(nb) // 256
    return ids


def _stepped_uniform(seed=61, wcorr=False):
    wl, ic, x, f = G.make_case(nb=(2, 3, 2), ppc=8, seed=seed, vscale=20.0)
    wc = None
    if wcorr:
        wc = np.random.default_rng(seed).uniform(0.5, 1.5, len(ic["spec"]))
    ctx = G.gpu_ctx(wl, ic, x, f, wcorr=wc)
    ctx.push_deposit()          # cells with arrivals: list order differs from import order
    ctx.push_deposit()
    wc_by_id = None if wc is None else wc.astype(np.float32).astype(np.float64)
    return ctx, wl, wc_by_id


@pytest.mark.parametrize("li", range(len(LAYOUTS)))
def test_uniform_section_bytes_and_checksum_match_oracle(li):
    layout = LAYOUTS[li]
    ctx, wl, wc = _stepped_uniform(wcorr=layout.off_weight >= 0)
    with ctx:
        nb = ctx.nblocks
        order = np.random.default_rng(3).permutation(nb).astype(np.int32)
        ids = _random_ids(nb, 12, 5)
        sec = ctx.write_restart_particles(layout, order, ids)
        exp = ctx.export_particles()
        x, v, sp, blk, cel, w = _oracle_inputs(exp, wc)
        ref = O.restart_pack(layout, nb, x, v, sp, blk, cel, [s.weight for s in wl.species], w, order, ids)
        assert sec.size == ref.size
        np.testing.assert_array_equal(sec, ref)
        for bo in (None, order):
            assert ctx.particle_checksum(layout, bo) == O.particle_checksum(layout, nb, x, v, sp, blk, cel,
                                                                            w, bo)


def test_amr_section_and_checksum_match_oracle():
    mesh, wl, ic, x, f = amr_case(ppc=8, seed=63, vscale=30.0)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.push_deposit()
        layout = RecordLayout.basic(False)
        nb = ctx.nblocks
        order = np.random.default_rng(4).permutation(nb).astype(np.int32)
        sec = ctx.write_restart_particles(layout, order)
        exp = ctx.export_particles()
        x_, v_, sp, blk, cel, _ = _oracle_inputs(exp)
        ref = O.restart_pack(layout, nb, x_, v_, sp, blk, cel, [s.weight for s in wl.species], None, order)
        np.testing.assert_array_equal(sec, ref)
        assert ctx.particle_checksum(layout, order) == O.particle_checksum(layout, nb, x_, v_, sp, blk, cel,
                                                                           None, order)
        # read back: the same lists, the same checksum and positions
        c0 = ctx.particle_checksum(layout)
        assert ctx.read_restart_particles(sec, layout) == exp["x"].shape[0]
        assert ctx.particle_checksum(layout) == c0
        e2 = ctx.export_particles(ids=False)
        for k in ("x", "v", "spec", "block", "cell"):
            np.testing.assert_array_equal(e2[k], exp[k])


@pytest.mark.parametrize("wcorr", [False, True])
def test_read_back_restores_lists_and_next_step(wcorr):
    layout = RecordLayout.basic(wcorr)
    ctx, wl, wc = _stepped_uniform(seed=65, wcorr=wcorr)
    with ctx:
        ids = _random_ids(ctx.nblocks, 12, 6)
        order = np.arange(ctx.nblocks, dtype=np.int32)[::-1].copy()
        sec = ctx.write_restart_particles(layout, order, ids)
        c0 = ctx.particle_checksum(layout)
        exp = ctx.export_particles(ids=False)
        fields = ctx.export_fields()
        # a fresh context of the same mesh reads the section
        cap = exp["x"].shape[0] + 4096
        with A.EcsimContext(wl, capacity=cap, track_ids=True) as ctx2:
            ctx2.import_fields(**fields)
            assert ctx2.read_restart_particles(sec, layout, ids) == exp["x"].shape[0]
            assert ctx2.particle_checksum(layout) == c0
            e2 = ctx2.export_particles()
            for k in ("x", "v", "spec", "block", "cell"):
                np.testing.assert_array_equal(e2[k], exp[k])
            # ids follow the section's order (the reference gives new particles new indices)
            assert sorted(e2["id"].tolist()) == list(range(exp["x"].shape[0]))
            # the section written again is the same bytes
            np.testing.assert_array_equal(ctx2.write_restart_particles(layout, order, ids), sec)
            # one more step from both states: the same particles (arrivals may
            # land in another order within a cell, so compare sorted sets) and
            # the same moments up to FP32 summation order
            ctx.push_deposit()
            ctx2.push_deposit()
            a, b = ctx.export_particles(ids=False), ctx2.export_particles(ids=False)

            def canon(e):
                k = np.lexsort((e["v"][:, 0], e["x"][:, 2], e["x"][:, 1], e["x"][:, 0],
                                e["cell"], e["block"]))
                return {q: e[q][k] for q in ("x", "v", "spec", "block", "cell")}
            a, b = canon(a), canon(b)
            for k in a:
                np.testing.assert_array_equal(a[k], b[k])
            J1, M1 = ctx.export_moments()
            J2, M2 = ctx2.export_moments()
            assert G.rel_err(J2, J1) <= 1e-6 and G.rel_err(M2, M1) <= 1e-6


def test_empty_and_single_particle_sections():
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=1, seed=67)
    layout = RecordLayout.basic(False)
    with A.EcsimContext(wl, capacity=4096, track_ids=True) as ctx:
        ctx.import_particles(x[:0], ic["v"][:0].astype(np.float64), ic["spec"][:0])
        sec = ctx.write_restart_particles(layout)
        assert sec.size == 43 + 8 + 8 * len(wl.species)
        assert ctx.particle_checksum(layout) == 0
        assert ctx.read_restart_particles(sec, layout) == 0
        ctx.import_particles(x[:1], ic["v"][:1].astype(np.float64), ic["spec"][:1])
        exp = ctx.export_particles()
        x1, v1, sp, blk, cel, _ = _oracle_inputs(exp)
        want = O.particle_checksum(layout, ctx.nblocks, x1, v1, sp, blk, cel)
        assert ctx.particle_checksum(layout) == want
        sec = ctx.write_restart_particles(layout)
        assert ctx.read_restart_particles(sec, layout) == 1
        assert ctx.particle_checksum(layout) == want


def test_malformed_sections_are_rejected():
    ctx, wl, _ = _stepped_uniform(seed=69)
    layout = RecordLayout.basic(False)
    with ctx:
        sec = ctx.write_restart_particles(layout)
        c0 = ctx.particle_checksum(layout)
        bad_marker = sec.copy()
        bad_marker[0] ^= 1
        with pytest.raises(AmpsGpuError):
            ctx.read_restart_particles(bad_marker, layout)
        with pytest.raises(AmpsGpuError):             # ParticleDataLength differs
            ctx.read_restart_particles(sec, RecordLayout.basic(True))
        with pytest.raises(AmpsGpuError):             # truncated records
            ctx.read_restart_particles(sec[:-1], layout)
        unknown = sec.copy()
        hdr = 43 + 8 + 8 * len(wl.species)
        unknown[hdr:hdr + 8] = np.frombuffer(np.int64(10 ** 9).tobytes(), np.uint8)
        with pytest.raises(AmpsGpuError):             # node id not in the mesh
            ctx.read_restart_particles(unknown, layout)
        # rejected sections leave the particles untouched
        assert ctx.particle_checksum(layout) == c0
        # a record moved into another cell's range is loaded clamped and reported
        moved = sec.copy()
        rec0 = hdr + 8 + 4 + 4 * 512
        xoff = rec0 + layout.off_position
        xv = moved[xoff:xoff + 8].view(np.float64).copy()
        moved[xoff:xoff + 8] = np.frombuffer((xv + 3.0 * wl.mesh.dx).tobytes(), np.uint8)
        with pytest.raises(AmpsGpuError, match="outside their cell"):
            ctx.read_restart_particles(moved, layout)
        assert ctx.num_particles() == ctx.export_particles()["x"].shape[0]


def test_checksum_at_size_matches_oracle():
    """a larger population: the chunked device combination over ~10^6 records"""
    wl, ic, x, f = G.make_case(nb=(4, 4, 4), ppc=32, seed=71, vscale=10.0)
    layout = RecordLayout.basic(False)
    with G.gpu_ctx(wl, ic, x, f) as ctx:
        ctx.push_deposit()
        exp = ctx.export_particles()
        x1, v1, sp, blk, cel, _ = _oracle_inputs(exp)
        assert x1.shape[0] > 10 ** 6
        assert ctx.particle_checksum(layout) == O.particle_checksum(layout, ctx.nblocks, x1, v1, sp, blk, cel)


def test_page_locked_buffers_give_the_same_section():
    """page-locked output is written and page-locked input read by the device in
    place; the bytes and the restored state equal those of pageable buffers"""
    ctx, wl, _ = _stepped_uniform(seed=73)
    layout = RecordLayout.basic(False)
    pin = A.PinnedArrays()
    try:
        with ctx:
            sec = ctx.write_restart_particles(layout)
            buf = pin.empty(sec.size + 100, np.uint8)
            buf[:] = 0xAB
            got = ctx.write_restart_particles(layout, out=buf)
            np.testing.assert_array_equal(got, sec)
            assert (buf[sec.size:] == 0xAB).all()
            c0 = ctx.particle_checksum(layout)
            exp = ctx.export_particles(ids=False)
            ctx.read_restart_particles(buf[:sec.size], layout)
            assert ctx.particle_checksum(layout) == c0
            e2 = ctx.export_particles(ids=False)
            for k in ("x", "v", "spec", "block", "cell"):
                np.testing.assert_array_equal(e2[k], exp[k])
    finally:
        pin.free()
