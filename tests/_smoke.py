"""One small simulate -> extract -> fit -> remove run on cuda:0, checked against the oracle
(used by __graft_entry__.smoke())."""
import numpy as np

from radiolensfit2_gb300 import _lib
from radiolensfit2_gb300.pipeline import DeviceObservation

import _oracle as O
from _cases import Case, oracle_sky_model, oracle_data_processing


def run():
    orc = O.load_oracle()
    case = Case(n_gal=4)
    sky = oracle_sky_model(orc, case)
    _, _, _, _, ref = oracle_data_processing(orc, case, case.data, sky)
    dev = DeviceObservation(case.obs, precision=_lib.RLF_F64, sigma2=case.sigma2, flag=case.flag)
    dev.set_vis(case.data, sky)
    pr = dev.process(case.cat, batch=1, refit=False)
    for gi, r in enumerate(ref):
        assert pr.results["error"][gi] == r[6], (gi, pr.results[gi], r)
        assert abs(pr.results["e1"][gi] - r[0]) < 1e-6 and abs(pr.results["e2"][gi] - r[1]) < 1e-6, (gi, pr.results[gi], r)
    dev.close()
    devm = DeviceObservation(case.obs, precision=_lib.RLF_MIXED, sigma2=case.sigma2, flag=case.flag)
    devm.set_vis(case.data, sky)
    pm = devm.process(case.cat, batch=4, refit=False)
    dmax = float(np.max(np.abs(pm.results["e1"] - np.array([r[0] for r in ref]))))
    print(f"smoke: F64 path matches the oracle on {case.cat.n} galaxies; mixed batched |de1|max={dmax:.2e}")
    devm.close()
