"""A father block with one refined son (ratio 2), stepped on the oracle and on
the GPU in the order of tree_collision_streaming_IBM_FEM
(LBMBlockComm.f90:279-318): father step with face extraction before and after
it, two son sub-steps each followed by the father-to-son face interpolation,
then the son-to-father injection."""
import numpy as np

import oracle as O

FATHER = dict(dims=(20, 12, 12), dh=1.0, origin=(0.0, 0.0, 0.0), bnd=(101, 104, 301, 301, 301, 301))
SON = dict(dims=(9, 7, 7), dh=0.5, origin=(6.0, 4.0, 4.0), bnd=(0, 0, 0, 0, 0, 0))


class TwoLevel:
    def __init__(self, gpu=True, scheme=1, model=1, nu=0.02, uvwIn=(0.05, 0.0, 0.0), precision=None):
        self.fl = O.make_flow(uvwIn=uvwIn, nu=nu, interpolateScheme=scheme)
        self.ofa = O.Block(*FATHER["dims"], FATHER["dh"], FATHER["origin"], list(FATHER["bnd"]), model, self.fl)
        self.oso = O.Block(*SON["dims"], SON["dh"], SON["origin"], list(SON["bnd"]), model, self.fl)
        self.opair = O.Pair(self.ofa, self.oso, scheme)
        self.time = 0.0
        self.gpu = gpu
        for b in (self.ofa, self.oso):
            b.initialise(0.0)
            b.set_bc()
        if gpu:
            import fsilbm3d_gb300 as F
            kw = dict(iCollidModel=model, nu=nu, precision=F.PREC_F64 if precision is None else precision,
                      uvwIn=uvwIn)
            self.gfa = F.Block(*FATHER["dims"], dh=FATHER["dh"], origin=FATHER["origin"], bndConds=FATHER["bnd"],
                               m_collid=self._m(self.ofa, "mc", model), m_force=self._m(self.ofa, "mf", model), **kw)
            self.gso = F.Block(*SON["dims"], dh=SON["dh"], origin=SON["origin"], bndConds=SON["bnd"],
                               m_collid=self._m(self.oso, "mc", model), m_force=self._m(self.oso, "mf", model), **kw)
            for b in (self.gfa, self.gso):
                b.initialise(0.0)
                b.set_boundary_conditions(0.0)
            self.gpair = F.Pair(self.gfa, self.gso, scheme)

    @staticmethod
    def _m(ob, key, model):
        if model != 3:
            return None
        return np.array(getattr(ob.b, key)[:]).reshape(19, 19, order="F")

    def step(self):
        self.time += FATHER["dh"]
        t = self.time
        self.ofa.b.blktime = t
        self.oso.b.blktime = t
        O.block_stage_pre(self.ofa)
        self.opair.extract(1)
        O.block_stage_post(self.ofa)
        self.opair.extract(2)
        for n in range(2):
            self.oso.b.blktime = self.oso.b.blktime + n * SON["dh"]
            O.block_stage_pre(self.oso)
            O.block_stage_post(self.oso)
            self.opair.father_to_son(n)
        self.opair.son_to_father()
        if self.gpu:
            z = (0.0, 0.0, 0.0)
            self.gpair.extract(1)
            self.gfa.step(z, t)
            self.gpair.extract(2)
            st = t
            for n in range(2):
                st = st + n * SON["dh"]
                self.gso.step(z, st)
                self.gpair.father_to_son(n, z)
            self.gpair.son_to_father(z)
