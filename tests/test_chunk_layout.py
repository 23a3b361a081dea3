"""Lane layout of the FP32 node kernels (the `Chunk` struct of kernels_fp32_batched.cu),
restated in Python and checked for every column height up to 128 layers: each layer of a
column is stored exactly once per tracer, by a lane whose vertical neighbours (the halo levels
the stage reads through shuffles) sit in the same segment, and no segment reaches past the
warp; the packed last chunk holds floor(32 / W) tracers."""
import pytest

HALOS = {"lo_ad": (2, 1), "bounds": (1, 1), "update": (1, 1)}


def chunk(nzmin, nzmax, ch, lane, HU, HD, W=32, P=1, packed=False):
    OUT = 32 - HU - HD
    if packed:
        q, l = lane // W, lane % W
        nz = nzmin - HU + OUT * ch + l
        lvl = q < P and nzmin <= nz <= nzmax - 1
        out = lvl and HU <= l < W - HD
    else:
        q, l = 0, lane
        nz = nzmin - HU + OUT * ch + lane
        lvl = nzmin <= nz <= nzmax - 1
        out = lvl and HU <= lane < 32 - HD
    return q, l, nz, lvl, out


def layout(nzmin, nzmax, HU, HD):
    """(tracer slot, nz, lane) of every stored lane, chunk by chunk, as the node kernels run."""
    OUT = 32 - HU - HD
    nl = nzmax - nzmin
    nch = (nl + OUT - 1) // OUT
    W = nl - OUT * (nch - 1) + HU + HD
    P = 32 // W
    stored = []
    for ch in range(nch):
        packed = ch == nch - 1 and P > 1
        for lane in range(32):
            q, l, nz, lvl, out = chunk(nzmin, nzmax, ch, lane, HU, HD, W, P, packed)
            if out:
                width = W if packed else 32
                stored.append((ch, q, nz, l, width))
    return stored, nch, W, P


@pytest.mark.parametrize("stage", sorted(HALOS))
@pytest.mark.parametrize("nzmin", [1, 3])
def test_every_layer_stored_once_with_its_halo_in_segment(stage, nzmin):
    HU, HD = HALOS[stage]
    for nlay in range(1, 129):
        nzmax = nzmin + nlay
        stored, nch, W, P = layout(nzmin, nzmax, HU, HD)
        assert 1 <= W <= 32
        last_packed = P > 1
        # every tracer runs the full chunks alone (slot 0) and the last chunk in some slot q
        full = [nz for ch, q, nz, l, w in stored if not (last_packed and ch == nch - 1)]
        for q in range(P if last_packed else 1):
            last = [nz for ch, qq, nz, l, w in stored if last_packed and ch == nch - 1 and qq == q]
            levels = full + last
            assert sorted(levels) == list(range(nzmin, nzmax)), (stage, nlay, q)
            assert len(set(levels)) == len(levels)
        for ch, q, nz, l, width in stored:
            # the shuffles a stored lane takes (HU up, HD down) stay inside its segment
            assert l - HU >= 0 and l + HD <= width - 1, (stage, nlay, ch, l, width)
            assert q * width + l < 32


def test_packing_factor_on_deep_columns():
    # 69 layers: chunks of 30, 30 and a last chunk of 9 levels + 2 halo lanes -> 2 tracers
    stored, nch, W, P = layout(1, 70, 1, 1)
    assert (nch, W, P) == (3, 11, 2)
    # lo_ad: chunks of 29, 29, 11 + 3 halo lanes -> 2 tracers
    stored, nch, W, P = layout(1, 70, 2, 1)
    assert (nch, W, P) == (3, 14, 2)
    # a 13-layer column: one chunk of 15 lanes -> 2 tracers side by side
    assert layout(1, 14, 1, 1)[1:] == (1, 15, 2)


def test_edge_passes_store_every_level_once():
    """k32_ho: passes of 32 levels over an edge's range [elo, ehi]; the last pass, when its W
    levels fill at most half a warp, carries floor(32 / W) tracers in segments of W lanes."""
    for elo in (1, 4):
        for nlev in range(1, 129):
            ehi = elo + nlev - 1
            per_tracer = {}
            nz0 = elo
            while nz0 + 32 <= ehi:  # full passes: one tracer per pass
                per_tracer.setdefault(0, []).extend(range(nz0, nz0 + 32))
                nz0 += 32
            W = ehi - nz0 + 1
            P = 32 // W
            for lane in range(32):
                q = lane // W if P > 1 else 0
                nz = nz0 + lane - q * W
                if nz <= ehi and q < P:
                    per_tracer.setdefault(q, [])
                    per_tracer[q].append(nz)
            full = [z for z in per_tracer.get(0, []) if z < nz0]
            for q in range(P):
                levels = full + [z for z in per_tracer.get(q, []) if z >= nz0]
                assert sorted(levels) == list(range(elo, ehi + 1)), (elo, nlev, q)
