"""The pipeline's flex_config-style settings (e8g_pipeline_config_set, host only): the reference's
names and defaults (pipeline.cpp:103-185) map onto the modes, layouts and compositor settings."""
import pytest

from x3dcore2_gb300 import abi
from x3dcore2_gb300.core import pipeline_config


def test_defaults_are_the_references(lib):
    c = pipeline_config()
    assert (c.mode, c.layout, c.samples_per_frame, c.firefly_filter, c.auto_exposure, c.exposure) == (
        abi.MODE_REF_UNI, abi.BVH_SAH, 64, 0, 0, 1.0)
    assert c.progressive == 0 and c.integrator == abi.INTEGRATOR_MEGAKERNEL


@pytest.mark.parametrize("name,mode", [
    ("normal", abi.MODE_NORMAL), ("position", abi.MODE_POSITION), ("direct", abi.MODE_REF_DIRECT),
    ("unidirectional", abi.MODE_REF_UNI), ("unidirectional_lt1", abi.MODE_REF_LT1),
    ("bidirectional_lt2", abi.MODE_REF_LT2), ("bidirectional_mis", abi.MODE_REF_BDPT),
    ("mis", abi.MODE_MIS), ("bidirectional_power", abi.MODE_BDPT_POWER)])
def test_path_tracer_names(lib, name, mode):
    assert pipeline_config(path_tracer=name).mode == mode


def test_other_settings(lib):
    c = pipeline_config(path_space="wide_bvh", samples_per_frame=16, firefly_filter=True, auto_exposure="1",
                        exposure="1.75", progressive=True, integrator="wavefront", seed=42, num_threads=3,
                        light_sources="basic", super_samples=4)
    assert (c.layout, c.samples_per_frame, c.firefly_filter, c.auto_exposure, c.exposure) == (
        abi.BVH_WIDE, 16, 1, 1, 1.75)
    assert (c.progressive, c.integrator, c.seed, c.num_threads) == (1, abi.INTEGRATOR_WAVEFRONT, 42, 3)
    assert pipeline_config(path_space="reference_bvh").layout == abi.BVH_REFERENCE
    assert pipeline_config(path_space="linear").layout == abi.BVH_LINEAR


@pytest.mark.parametrize("key,value,status", [
    ("path_tracer", "photon_mapping", "INVALID_ARG"),
    ("path_space", "kd_tree", "INVALID_ARG"), ("samples_per_frame", "0", "INVALID_ARG"),
    ("samples_per_frame", "-3", "INVALID_ARG"), ("exposure", "bright", "INVALID_ARG"),
    ("auto_exposure", "maybe", "INVALID_ARG"), ("light_sources", "sky", "INVALID_ARG"),
    ("scene_file", "cornellball", "INVALID_ARG"), ("integrator", "photon", "INVALID_ARG")])
def test_refused_settings(lib, key, value, status):
    with pytest.raises(abi.E8GError, match=status):
        pipeline_config(**{key: value})
