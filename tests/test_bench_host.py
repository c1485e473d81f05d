"""CPU tests of bench.py's host-side pieces.  The split/merge section runs end to end with
the device entry points answered by the oracle, so its host leg (the two searches of the
oracle port, the timings and the bit-for-bit checks) and the JSON it builds are exercised
without a GPU."""
import json

import numpy as np

import oracle as O


class _HostTensor:
    """Stands in for a device tensor: a numpy array with clone(), cpu(), numpy() and to()."""

    def __init__(self, a):
        self.a = np.ascontiguousarray(a)

    def clone(self):
        return _HostTensor(self.a.copy())

    def cpu(self):
        return self

    def numpy(self):
        return self.a

    def to(self, dev):
        return self


class _HostTorch:
    class cuda:
        @staticmethod
        def synchronize():
            pass

        @staticmethod
        def current_device():
            return 0

    @staticmethod
    def device(*args):
        return None

    @staticmethod
    def from_numpy(a):
        return _HostTensor(a)


class _OracleG:
    """split_elongated / merge_close_particles with the package's call surface, answered by
    the oracle in index order (what the kernels compute)."""

    @staticmethod
    def split_elongated(x, s, r, e, core, overlap, threshold):
        out = O.split_elongated(x.a, s.a, r.a, e.a, {"gaussian": 0, "compactg": 1}[core], overlap, threshold)
        return tuple(_HostTensor(v) for v in out[:4]) + (out[4],)

    @staticmethod
    def merge_close_particles(x, s, r, overlap, threshold, adapt):
        out = O.merge_close_particles(x.a, s.a, r.a, overlap, threshold, adapt)
        return tuple(_HostTensor(v) for v in out[:3]) + (out[3],)


def test_splitmerge_section_on_host():
    import bench
    from omega3d_gb300 import workloads as W
    out = bench.bench_splitmerge(None, _OracleG, _HostTorch, W, reps=1, k=12)
    json.dumps(out)
    assert out["particles"] == 12 ** 3
    assert out["split"]["nsplit"] > 0 and out["merge"]["nremoved"] > 0
    for op in ("split", "merge"):
        d = out[op]
        assert d["bit_identical_to_port"] is True
        assert d["port_kdtree_equals_cell_list"] is True
        assert d["ms"] > 0 and d["cpu_port_ms"] > 0 and d["cpu_port_cell_list_ms"] > 0
    assert out["cpu_port"]["cores"] == 1 and "kd-tree" in out["cpu_port"]["sample"]


def test_cpu_splitmerge_orders_agree_without_ties():
    import bench
    from omega3d_gb300 import workloads as W
    x, s, r, e = W.lattice_particles(k=16, seed=41)
    res = bench.cpu_splitmerge(x, s, r, e)
    assert set(res) == {"kdtree", "index"}
    (ks, _, km, _), (cs, _, cm, _) = res["kdtree"], res["index"]
    assert ks[4] == cs[4] > 0 and km[3] == cm[3] > 0
    for a, b in zip(ks[:4] + km[:3], cs[:4] + cm[:3]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_guarded_section_reports_errors_in_the_line():
    import bench
    assert bench.guarded(lambda: {"ms": 1.0}) == {"ms": 1.0}

    def broken():
        raise RuntimeError("o3g_batch_run failed: timeout")

    out = bench.guarded(broken)
    assert out == {"error": "RuntimeError: o3g_batch_run failed: timeout"}
    json.dumps(out)


def test_bem_rates_are_the_algorithmic_figures():
    """The BEM section's assembly rate counts the matrix written once (4 n^2 bytes) and the
    factorisation's effective rate 2/3 n^3 flops."""
    import bench
    r = bench.bem_rates(40960, 8.0, 280.0)
    assert abs(r["assemble_gbs"] - 4.0 * 40960 ** 2 / 8.0e-3 / 1e9) < 1e-9
    assert abs(r["factor_tflops_effective"] - (2.0 / 3.0) * 40960.0 ** 3 / 0.28 / 1e12) < 1e-9
    pk = bench.measured_peaks()
    if pk.get("hbm_gbs"):
        assert abs(r["assemble_frac_of_hbm"] - r["assemble_gbs"] / pk["hbm_gbs"]) < 1e-12
