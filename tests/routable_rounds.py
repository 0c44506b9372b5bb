"""The oracle's side of the routability-driven rounds (test infrastructure):
the rounds of texo_gb300.routability.place_routable run by the FP64 oracle,
with its FP64 RUDY map and register-clustering areas in the proposal, and
the two-kind routability case both sides are run on."""
import numpy as np

from oracle import ffi

from rich_problems import rich_problem


class OracleRounds:
    def __init__(self, problem, params, threads=5):
        self.o = ffi.Oracle(problem, params)
        self.threads = threads

        def demand(w, h, boxes):
            hd, vd, ok = ffi.routing_demand(w, h, boxes)
            assert ok
            return hd, vd

        def clustering(xy, clock_lsr, ce, count):
            code, areas = ffi.register_clustering_areas(xy, clock_lsr, ce, count)
            assert code == 0
            return areas
        self.demand, self.clustering = demand, clustering

    def fillers(self):
        f, q, _ = self.o.fillers()
        return f, q

    def round(self, stop, reset, scales, completed, coordinates):
        st, t, c, _, res = self.o.place_round(stop, reset, scales, completed, coordinates, threads=self.threads)
        return st, t, c, res

    def set_charges(self, member_charge, filler_charge):
        self.o.set_charges(member_charge, filler_charge)


def routability_case(seed=0, band=(22, 24), h_cap=6, v_cap=6):
    """The two-field (LUT + register) 2,000-cell problem with a routing
    capacity map whose horizontal channels are blocked in a band of rows (a
    hotspot that drives area inflation), and two register control sets (by
    clock). On the oracle: one area round installed (+121 % member area), a
    second proposal that grows nothing, and the final round, which the
    register field (its area inflated to fill the free capacity) reaches
    only at 222 iterations in all, with overflow 0.0999."""
    prob = rich_problem(seed)
    side = prob.width
    cap_h = np.full((side, side), h_cap, np.uint32)
    cap_v = np.full((side, side), v_cap, np.uint32)
    cap_h[band[0]:band[1], :] = 0
    regs = [int(prob.member_cell[i]) for i in range(len(prob.member_field)) if prob.member_field[i] == 1]
    controls = {c: (c % 2, 0, 0) for c in regs}
    return prob, cap_h, cap_v, controls
