"""bench.py's host-side helpers (CPU): the compact form summary that ends the
bench line, and the config both arms print for a workload."""
import importlib.util
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("mlem_bench", ROOT / "bench.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b


def test_forms_summary_headlines_and_ratios():
    b = _bench()
    forms = {
        "fp16_trans": {"images_iterations_per_s": 480.0},
        "fp32_plain_cyl3d_mid": {"images_iterations_per_s": 1750.0},
        "fp32_plain_ring2d": {"images_iterations_per_s": 110000.0},
        "batched_fp16_64": {"images_iterations_per_s": 8600.0, "sequential_fp32_images_iterations_per_s": 1760.0,
                            "vs_sequential_fp32": 8600.0 / 1760.0, "persistent_images_iterations_per_s": 7400.0,
                            "graphs_images_iterations_per_s": 8600.0},
        "modes_cyl3d_mid": {"csr_vector_trans": {"iterations_per_s": 1750.0},
                            "csr_vector_scatter": {"iterations_per_s": 1400.0}},
        "serving": {"requests": 2000, "p50_latency_s": 0.0123456, "p99_latency_s": 2.3, "reconstructions_per_s": 49.0,
                    "serial_fp32_reconstructions_per_s": 23.5, "vs_serial_fp32": 2.085, "p99_tail_samples": 20,
                    "mix": "not in the summary"},
        "symmetry": {"fp32": {"autotuned": {"iterations_per_s": 1290.0}}},
        "fused_pass": {"iterations_per_s": 289.0, "vs_fp32_plain": 289.0 / 268.0, "form": {"kernel": "rescan"}},
    }
    s = b.forms_summary(forms, 268.0)
    assert s["fused_pass_iter_s"] == 289.0 and s["fused_pass_vs_fp32_plain"] == round(289.0 / 268.0, 3)
    assert s["fp32_plain_iter_s"] == 268.0
    assert s["fp16_d16_images_iter_vs_fp32_plain"] == round(480.0 / 268.0, 3)
    assert s["batched_fp16_64_images_iter_vs_fp32_plain"] == round(8600.0 / 1750.0, 3)
    assert s["batched_vs_sequential_fp32"] == round(8600.0 / 1760.0, 3)
    assert s["mid_csr_vector_scatter_iter_s"] == 1400.0 and "mid_merge_trans_iter_s" not in s
    assert s["serving"]["p50_latency_s"] == 0.0123 and "mix" not in s["serving"]
    assert s["symmetry_matrix_hat_fp32_iter_s"] == 1290.0
    # empty forms: only the FP32 figure
    assert b.forms_summary({}, 100.0) == {"fp32_plain_iter_s": 100.0}


def test_both_arms_print_the_same_config():
    b = _bench()
    ours = b.workload_config("cyl3d_12gb", 2653056, 2560000, 1434025752, 1)
    ref = b.workload_config("cyl3d_12gb", 2653056, 2560000, 1434025752, 1)
    assert ours == ref and ours["values"] == "f32" and "L2" in ours["l2"]
    assert b.workload_config("ring2d", 1, 1, 1, 2, "f16")["values"] == "f16"
