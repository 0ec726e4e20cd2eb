"""Frame export and diagnostics on the GPU against what the reference
itself wrote and computed for the same state (tests/golden/frames_*.npz):
shear_sim::output / write_files byte for byte, qs_measure, tractions and
compute_strain to 1e-12."""
import numpy as np
import pytest

from stz_gb300.shear_sim import ShearSim

pytestmark = pytest.mark.gpu


def load_state(P, meta, ref):
    sim = ShearSim(P, ref["chi0"])
    for k in ("p", "q", "s", "tau", "chi", "X", "Y", "u", "v"):
        sim.set(k, ref[k])
    sim.time = meta["time"]
    return sim


def test_output_bytes_match_reference(golden_frames, tmp_path):
    name, P, meta, ref = golden_frames
    with load_state(P, meta, ref) as sim:
        for mode in range(11):
            got = sim.output(mode)
            assert got.shape == ref[f"output{mode}"].shape, mode
            np.testing.assert_array_equal(got, ref[f"output{mode}"], err_msg=f"mode {mode}")
        qs = sim.write_files(tmp_path, 7, flags=(1 << 12) - 1)
        for mode, prefix in enumerate(["u", "v", "p", "q", "s", "tau", "chi", "tem", "dev", "X", "Y"]):
            assert (tmp_path / f"{prefix}.7").read_bytes() == ref[f"output{mode}"].tobytes(), prefix
        np.testing.assert_allclose(qs, ref["qs"], rtol=1e-12)
        proj = np.fromfile(tmp_path / "proj.7", dtype=np.float32).reshape(ref["output11"].shape)
        np.testing.assert_allclose(proj, ref["output11"], rtol=1e-6)


def test_diagnostics_match_reference(golden_frames):
    name, P, meta, ref = golden_frames
    with load_state(P, meta, ref) as sim:
        np.testing.assert_allclose(sim.qs_measure(False), ref["qs"], rtol=1e-12)
        np.testing.assert_allclose(sim.qs_measure(True), ref["qs_staggered"], rtol=1e-12)
        t = ref["tractions"]
        np.testing.assert_allclose(sim.tractions(), t, rtol=1e-12, atol=1e-14 * np.abs(t).max())
        st = sim.compute_strain()
        np.testing.assert_allclose(st, ref["strain"], rtol=1e-12, atol=1e-14)
        assert np.all(st[1:-1] == 0) and np.all(st[0] > 0)
