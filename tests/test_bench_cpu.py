"""bench.py on the CPU: its work models, and the reference arm's JSON line
(the C++ restatement of the walker step timed on the host cores, with its
calibration against the reference's published per-core rate) on the smallest
workload."""
import json
import os
import subprocess
import sys

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_work_models_cover_the_timed_stages():
    fl = bench.flops_model(120, 20, 20, 600)
    for k in ("fb", "vhs", "prop", "overlap", "ortho", "energy"):
        assert fl[k] > 0
    assert fl["step"] == fl["fb"] + fl["vhs"] + fl["prop"] + fl["overlap"] + fl["ortho"]
    pipes = bench.mixed_stage_pipes(120, 20, 20, 600)
    assert set(pipes) == {"vhs", "prop", "overlap", "ortho"}
    for parts in pipes.values():
        for name, flops, pipe, cost in parts:
            assert flops > 0 and cost >= 1 and pipe in ("tensor", "fp32"), name
    # the tensor-core stages carry the algorithmic FLOPs of the headline roofline
    assert pipes["prop"][0][1] == fl["prop"] and pipes["vhs"][0][1] == fl["vhs"]
    assert 70 < bench.fp32_nominal_tflops() < 90


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "cfg1", "--steps", "2",
                        "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "walker-steps/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["n_gpus"] == 1
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "walker-steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cal = cb["calibration"]
    assert cal["port_per_core"] > 0 and abs(cal["reference_published_per_core"] - 37277.0) < 1.0


def _undefined_globals(path):
    """Names a function of the module reads as globals that the module never
    binds (assignment, import, def or class) and that are not builtins."""
    import builtins
    import symtable
    top = symtable.symtable(open(path).read(), path, "exec")
    bound = {s.get_name() for s in top.get_symbols() if s.is_assigned() or s.is_imported() or s.is_namespace()}
    bound |= {"__file__", "__name__", "__doc__", "__spec__", "__loader__", "__package__"}
    bad = set()

    def walk(t):
        for s in t.get_symbols():
            n = s.get_name()
            if s.is_global() and s.is_referenced() and n not in bound and not hasattr(builtins, n):
                bad.add(n)
        for c in t.get_children():
            walk(c)

    walk(top)
    return bad


def test_no_undefined_globals():
    """Code paths that only run on a GPU (bench.py's main, the package's
    launchers) are not executed by the CPU suite; this catches a name they use
    that no longer exists."""
    files = [os.path.join(ROOT, "bench.py"), os.path.join(ROOT, "__graft_entry__.py")]
    pkg = os.path.join(ROOT, "vmc_gb300")
    files += [os.path.join(pkg, f) for f in sorted(os.listdir(pkg)) if f.endswith(".py")]
    for f in files:
        assert not _undefined_globals(f), (f, _undefined_globals(f))
