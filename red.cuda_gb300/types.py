"""Host-side records that mirror red.type/red_type.h, and the System container.

VAR4   var4_t                      red_type.h:206-212   32 bytes
PARAM  pp_disk_t::param_t          red_type.h:347-353   32 bytes
BMD    pp_disk_t::body_metadata_t  red_type.h:356-362   24 bytes (LP64 padding)
GAS    analytic_gas_disk_params_t  red_type.h:464-485  160 bytes
EVENT  pp_disk_t::event_data_t     red_type.h:415-461  432 bytes
"""
import numpy as np

VAR4 = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("w", "<f8")])
PARAM = np.dtype([("mass", "<f8"), ("radius", "<f8"), ("density", "<f8"), ("cd", "<f8")])
BMD = np.dtype({"names": ["id", "body_type", "mig_type", "mig_stop_at"],
                "formats": ["<i4", "<i4", "<i4", "<f8"],
                "offsets": [0, 4, 8, 16], "itemsize": 24})
GAS = np.dtype({"names": ["rho", "sch", "eta", "tau", "mfp", "temp", "c_vth", "gas_decrease",
                          "t0", "t1", "e_folding_time", "alpha", "mean_molecular_weight",
                          "particle_diameter"],
                "formats": [("<f8", 2)] * 6 + ["<f8", "<i4"] + ["<f8"] * 6,
                "offsets": [0, 16, 32, 48, 64, 80, 96, 104, 112, 120, 128, 136, 144, 152],
                "itemsize": 160})
EVENT = np.dtype({"names": ["event_name", "t", "d",
                            "id0", "idx0", "p0", "r0", "v0",
                            "id1", "idx1", "p1", "r1", "v1",
                            "id2", "idx2", "p2", "r2", "v2",
                            "ps", "rs", "vs"],
                  "formats": ["<i4", "<f8", "<f8",
                              "<i4", "<u4", PARAM, VAR4, VAR4,
                              "<i4", "<u4", PARAM, VAR4, VAR4,
                              "<i4", "<u4", PARAM, VAR4, VAR4,
                              PARAM, VAR4, VAR4],
                  "offsets": [0, 8, 16, 24, 28, 32, 64, 96, 128, 132, 136, 168, 200,
                              232, 236, 240, 272, 304, 336, 368, 400],
                  "itemsize": 432})

# body types, red_type.h:169-179
STAR, GIANTPLANET, ROCKYPLANET, PROTOPLANET, SUPERPLANETESIMAL, PLANETESIMAL, TESTPARTICLE = range(7)
# integrator types, red_type.h:136-143
EULER, RUNGEKUTTA2, RUNGEKUTTA4, RUNGEKUTTAFEHLBERG56, RUNGEKUTTAFEHLBERG78 = range(5)
# event names, red_type.h:145-152
EVENT_NONE, EVENT_HIT_CENTRUM, EVENT_EJECTION, EVENT_COLLISION = range(4)
# gas density time dependence, red_type.h:105-111
GAS_DENSITY_CONSTANT, GAS_DENSITY_DECREASE_LINEAR, GAS_DENSITY_DECREASE_EXPONENTIAL = range(3)


class System:
    """One red system on the host: r, v (var4), p (param), md (metadata) and the
    number of bodies per type (n_objects_t::playing), bodies sorted by type."""

    def __init__(self, r, v, p, md, playing, names=None):
        self.r = np.ascontiguousarray(r, dtype=VAR4)
        self.v = np.ascontiguousarray(v, dtype=VAR4)
        self.p = np.ascontiguousarray(p, dtype=PARAM)
        self.md = np.ascontiguousarray(md, dtype=BMD)
        self.playing = np.ascontiguousarray(playing, dtype=np.uint32)
        self.inactive = np.zeros(7, np.uint32)
        self.removed = np.zeros(7, np.uint32)
        self.names = names

    @property
    def n(self):
        return int(self.playing.sum())

    @property
    def n_SI(self):
        return int(self.playing[:4].sum())

    @property
    def n_NSI(self):
        return int(self.playing[4:6].sum())

    @property
    def n_NI(self):
        return int(self.playing[6])

    def active_counts(self):
        return (self.playing - self.inactive).astype(np.uint32)

    def copy(self):
        s = System(self.r.copy(), self.v.copy(), self.p.copy(), self.md.copy(), self.playing.copy(),
                   None if self.names is None else list(self.names))
        s.inactive = self.inactive.copy()
        s.removed = self.removed.copy()
        return s

    def interactions_per_eval(self):
        nsi, nnsi, nni = self.n_SI, self.n_NSI, self.n_NI
        nm = nsi + nnsi
        return (nsi * (nm - 1) if nsi else 0) + nnsi * nsi + nni * nm

    def relabel_all_SI(self):
        """The dense variant: every planetesimal becomes a protoplanet (type 3),
        so every massive pair interacts.  A legal red input."""
        s = self.copy()
        nsi, nnsi = self.n_SI, self.n_NSI
        s.md["body_type"][nsi:nsi + nnsi] = PROTOPLANET
        pl = s.playing.copy()
        pl[PROTOPLANET] += pl[SUPERPLANETESIMAL] + pl[PLANETESIMAL]
        pl[SUPERPLANETESIMAL] = 0
        pl[PLANETESIMAL] = 0
        s.playing = pl
        return s
