"""Host-side logic that needs no GPU: namelist and model.h readers, the
memchunk time interpolation, case files, the synthetic workloads, and
bench.py's reading of the committed step-kernel profile."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

from swm_gb300.host import caseio, memchunk, modelh, namelist, synthetic


def test_namelist_groups_values_and_comments():
    text = """
    ! a comment line
    &model_nl
      dt = 1.5d2, run_length=3600 ! trailing comment
      file_name = 'a!b.nc'
      flag = .TRUE.
    /
    &swm_damping_nl gamma_new=1e-5, gamma_new_sponge = 2.0E-4 /
    &swm_damping_nl gamma_new=3e-5 /
    &arrays x = 1, 2, 3 /
    """
    g = namelist.parse(text)
    m = namelist.group(g, 'MODEL_NL')
    assert m['dt'] == 150.0 and m['run_length'] == 3600
    assert m['file_name'] == 'a!b.nc' and m['flag'] is True
    damp = namelist.groups_named(g, 'swm_damping_nl')
    assert [d['gamma_new'] for d in damp] == [1e-5, 3e-5]
    assert damp[0]['gamma_new_sponge'] == 2e-4
    assert namelist.group(g, 'arrays')['x'] == [1, 2, 3]
    assert namelist.group(g, 'missing') == {}


def test_model_h_defines_outside_comments():
    text = """
    #define FULLY_NONLINEAR
    /* #define LATERAL_MIXING
       still a comment */
    #define TAU_SCALE 1.5
    """
    d = modelh.parse_defines(text)
    assert 'FULLY_NONLINEAR' in d and 'LATERAL_MIXING' not in d
    assert d['TAU_SCALE'] == '1.5'


def test_memchunk_linear_interpolation_and_cyclic_wrap():
    recs = np.arange(3, dtype=float)[:, None, None] * np.ones((3, 2, 2))  # values 0, 1, 2
    mc = memchunk.MemChunk(recs, dt_file=10.0, chunksize=100)
    assert mc.get(0.0)[0, 0] == 0.0
    assert mc.get(5.0)[0, 0] == pytest.approx(0.5)
    assert mc.get(20.0)[0, 0] == 2.0
    # the dataset repeats: record 3 (t = 30) is record 0 again
    assert mc.get(25.0)[0, 0] == pytest.approx(1.0)
    assert mc.get(30.0)[0, 0] == pytest.approx(0.0)
    const = memchunk.MemChunk(np.full((1, 2, 2), 7.0), dt_file=0.0, chunksize=10)
    assert const.is_constant and const.get(1e9)[1, 1] == 7.0


def test_memchunk_small_chunks_match_one_large_chunk():
    rng = np.random.default_rng(0)
    recs = rng.standard_normal((7, 3, 4))
    big = memchunk.MemChunk(recs, 4.0, 100)
    small = memchunk.MemChunk(recs, 4.0, 3)
    for t in np.arange(0.0, 60.0, 1.5):
        np.testing.assert_allclose(small.get(t), big.get(t), rtol=0, atol=1e-14)


def test_case_file_round_trip(tmp_path):
    case = synthetic.double_gyre((24, 16), biharmonic=True, nsteps=5)
    p = tmp_path / 'case.npz'
    caseio.save_case(str(p), case, extra_arrays={'note': np.arange(3)})
    back, extra = caseio.load_case(str(p))
    np.testing.assert_array_equal(extra['note'], np.arange(3))
    assert back['config'] == case['config']
    np.testing.assert_array_equal(back['H'], case['H'])
    assert len(back['streams']) == 1
    np.testing.assert_array_equal(back['streams'][0]['rec1'], case['streams'][0]['rec1'])


def test_double_gyre_time_step_inside_ab3_stability():
    """2*sqrt(2)*sqrt(gH)*dt/dx must stay below AB3's 0.72 on the imaginary axis."""
    case = synthetic.double_gyre(64, nsteps=1)
    cfg = case['config']
    c = np.sqrt(cfg['G'] * case['H'].max())
    assert 2 * np.sqrt(2) * c * cfg['dt'] / 5e3 < 0.72


def test_perturbed_basin_is_closed_with_bounded_inset():
    H = synthetic.perturbed_basin(40, 30, 500.0, np.random.default_rng(1), max_inset=3)
    assert (H[0] == 0).all() and (H[-1] == 0).all() and (H[:, 0] == 0).all() and (H[:, -1] == 0).all()
    assert (H[4:-4, 4:-4] == 500.0).all()


def test_bench_reads_the_step_kernels_traffic_from_their_profiles():
    """bench.py's roofline.traffic comes from the committed ncu summaries of
    the step kernels: the batched ensemble kernel (the headline) and the
    single-basin kernel; each must be there and parse, and lie between the
    kernel's written bytes and twice its algorithmic bytes (89 B per
    point)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location('bench_mod', os.path.join(ROOT, 'bench.py'))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    t = bench.profiled_traffic('k_march_double_gyre_1024.md')
    assert t is not None
    assert 20e6 < t < 2 * 89 * 1025 * 1025
    t = bench.profiled_traffic('k_march_ens_ensemble_256.md')
    assert t is not None
    assert 0.3 * 89 * bench.ENSEMBLE_256_POINTS < t < 2 * 89 * bench.ENSEMBLE_256_POINTS
