"""Batched path with its sub-batches captured as CUDA graphs (rlf_options.graphs = 1) against the
oracle's data_processing, and against the same path launched kernel by kernel: both passes, three
rounds with the device round control (a sub-batch whose fits stop changing skips its remaining
rounds on the GPU).  Tolerance of the batched FP32 path: |de| <= 1e-4 against the oracle."""
import numpy as np
import pytest

from radiolensfit2_gb300 import _lib
from radiolensfit2_gb300.pipeline import DeviceObservation

import _oracle as O
from _cases import Case, oracle_sky_model, oracle_data_processing

pytestmark = pytest.mark.gpu


def test_graph_capture_matches_oracle_and_direct_launches():
    orc = O.load_oracle()
    case = Case(n_ant=40, n_gal=14, fmin=30.0, fmax=200.0, noise=900.0, flag_frac=0.02)
    sky = oracle_sky_model(orc, case)
    _, _, _, _, ref = oracle_data_processing(orc, case, case.data, sky)
    err_ref = np.array([r[6] for r in ref])
    e_ref = np.array([(r[0], r[1]) for r in ref])
    dev = DeviceObservation(case.obs, precision=_lib.RLF_MIXED, sigma2=case.sigma2, flag=case.flag)
    dev.set_vis(case.data, sky)
    dev.snapshot()
    out = {}
    for graphs in (0, 1):
        dev.restore()
        pr = dev.process(case.cat, batch=6, refit=False, rounds=3, graphs=graphs)
        out[graphs] = pr
        good = err_ref == 0
        assert np.array_equal(pr.results["error"], err_ref), graphs
        de = np.maximum(np.abs(pr.results["e1"] - e_ref[:, 0]), np.abs(pr.results["e2"] - e_ref[:, 1]))[good]
        print(f"graphs={graphs}: |de| max {de.max():.2e}; stats {pr.stats}")
        assert de.max() < 1e-4
    d_g, s_g = dev.get_vis()
    dev.close()
    assert out[1].stats["graphs"] >= 2 and out[0].stats["graphs"] == 0
    for k in ("extract_passes", "extract_gal", "fitted", "remove_batches"):
        assert out[0].stats[k] == out[1].stats[k], k
    assert np.max(np.abs(out[1].results["e1"] - out[0].results["e1"])) < 1e-6
