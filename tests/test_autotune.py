"""Host logic of the tile-size / precision tuner of the batched mixed solver (CPU, no GPU):
re-tiling a batch between tile sizes against the oracle's own tile layout, and the selection
rule (the fastest candidate whose every matrix met the tolerance)."""
import numpy as np
import pytest

import oracle
from ttg_gb300 import autotune, batched_tile_offsets


def _batch_tiles(mats, NB):
    off, total = batched_tile_offsets([m.shape[0] for m in mats], NB)
    out = np.zeros(total)
    for k, A in enumerate(mats):
        t = oracle.tiles_from_full(A, NB)
        out[int(off[k]):int(off[k]) + t.size] = t
    return out


@pytest.mark.parametrize("nb_from,nb_to", [(256, 512), (512, 256), (128, 384)])
def test_retile_matches_the_tile_layout(gbx, nb_from, nb_to):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    sizes = [700, 256, 1300, 90, 513]
    mats = []
    for n in sizes:
        M = rng.standard_normal((n, n))
        mats.append((M + M.T) / 2)
    src = torch.from_numpy(_batch_tiles(mats, nb_from))
    got = autotune.retile(src, sizes, nb_from, nb_to).numpy()
    off, total = batched_tile_offsets(sizes, nb_to)
    assert got.size == total
    for k, n in enumerate(sizes):
        nt = (n + nb_to - 1) // nb_to
        t = got[int(off[k]):int(off[k]) + nt * (nt + 1) // 2 * nb_to * nb_to]
        assert np.array_equal(oracle.tiles_to_lower(t, n, nb_to), np.tril(mats[k]))
    back = autotune.retile(torch.from_numpy(got), sizes, nb_to, nb_from).numpy()
    off1, _ = batched_tile_offsets(sizes, nb_from)
    for k, n in enumerate(sizes):
        nt = (n + nb_from - 1) // nb_from
        t = back[int(off1[k]):int(off1[k]) + nt * (nt + 1) // 2 * nb_from * nb_from]
        assert np.array_equal(oracle.tiles_to_lower(t, n, nb_from), np.tril(mats[k]))


def test_select_mixed_takes_the_fastest_converged_candidate():
    table = {("fp16", 512, 0): (90.0, 0, 5e-15), ("bf16", 512, 0): (80.0, 0, 2e-14),   # too inaccurate
             ("fp8", 512, 1): (70.0, -4, 5e-15),                                       # did not converge
             ("fp16", 256, 0): (85.0, 0, 9e-15), ("fp16", 256, 1): (84.0, 0, 9e-15),
             ("bf16", 256, 1): (95.0, 0, 4e-15)}
    calls = []

    def run(prec, nb, sched):
        calls.append((prec, nb, sched))
        ms, st, be = table[(prec, nb, sched)]
        return {"ms": ms, "status": st, "backward_error_max": be}

    best = autotune.select_mixed(run, list(table), 1e-14)
    assert (best["prec"], best["NB"], best["sched"], best["ms"]) == ("fp16", 256, 1, 84.0)
    assert calls == list(table) and len(best["candidates"]) == len(table)
    assert [c["ok"] for c in best["candidates"]] == [True, False, False, True, True, True]
    with pytest.raises(RuntimeError):
        autotune.select_mixed(run, [("bf16", 512, 0), ("fp8", 512, 1)], 1e-14)
