"""Life B3/S23 on implicit raster edges (connect_raster_neighbors! with the
Moore neighbourhood, src/Raster.jl:139-167): the four-cells-per-word kernel
(raster widths divisible by 4) against the oracle's C restatement, periodic
and bounded, for widths that fill whole warps, leave a partial warp, or fit
in one word, and heights below and above a thread's row block."""
import numpy as np
import pytest

from oracle import models as om

pytestmark = pytest.mark.gpu

SIZES = [(128, 40), (132, 37), (4, 5), (8, 3), (1024, 64), (260, 9), (12, 1)]


def _life_sim(vh, W, H, periodic, alive):
    m = (vh.ModelTypes()
         .register_agenttype("Cell", [("alive", "bool")], ":Immortal")
         .register_edgetype("Neighbor", [], ":Stateless", target="Cell")
         .create_model("life_test"))
    sim = vh.create_simulation(m)
    vh.add_raster(sim, "raster", (W, H), "Cell", alive=alive)
    vh.connect_raster_neighbors(sim, "raster", "Neighbor", implicit=True, periodic=periodic)
    vh.finish_init(sim)
    return m, sim


@pytest.mark.parametrize("W,H", SIZES)
@pytest.mark.parametrize("periodic", [True, False])
def test_life_matches_oracle(vh, W, H, periodic):
    if periodic and H < 3:
        pytest.skip("a periodic dimension below 3 cells wraps onto the cell itself")
    rng = np.random.default_rng(W * 1000 + H)
    alive = rng.random(W * H) < 0.35
    m, sim = _life_sim(vh, W, H, periodic, alive)
    ref = alive.astype(np.uint8)
    for step in range(6):
        vh.apply_(sim, "life", ["Cell"], ["Cell", "Neighbor"], ["Cell"],
                  params=[m["Neighbor"].index])
        ref = om.life_step(ref, W, H, periodic=periodic)
        got = vh.read_agents(sim, "Cell")[0]["alive"].astype(np.uint8)
        np.testing.assert_array_equal(got, ref, err_msg="step %d" % step)
    sim.close()
