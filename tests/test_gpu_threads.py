"""Re-entrancy per host thread (the contract of src/libcusna.h: synchronous,
blocking calls; each host thread has its own stream, events and device
arena). Calls made from several threads at once, on problems of different
sizes and launch shapes (so different dynamic shared memory per launch),
return exactly what the same calls return one at a time."""
import concurrent.futures as cf

import numpy as np
import pytest

from cusna_gb300 import workloads as WL
from tests.golden.make_golden import run_case
from tests.test_gpu_parity import GpuEngine

pytestmark = pytest.mark.gpu

CASES = [("covariate", 5, 4, 1), ("structural", 33, 6, 2), ("coevol", 64, 5, 4),
         ("covariate_all", 97, 8, 1), ("interaction", 40, 6, 2), ("baseline", 200, 12, 8),
         ("masks", 70, 6, 4), ("gw", 50, 6, 2)]


def simulate(spec):
    kind, n, M, G = spec
    c = WL.parity_case(kind, seed=n + M, n=n, M=M)
    return run_case(GpuEngine(warps_per_chain=G, chains_per_cta=1), c)


def test_gpu_concurrent_calls_equal_serial_calls(gpu_lib):
    specs = [s for s in CASES if s[0] in WL.PARITY_KINDS]
    assert len(specs) >= 6
    serial = [simulate(s) for s in specs]
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        for rep in range(3):
            for spec, want, got in zip(specs, serial, ex.map(simulate, specs)):
                assert set(got) == set(want)
                for key in want:
                    np.testing.assert_array_equal(got[key], want[key],
                                                  err_msg=f"rep {rep}: {spec}: {key}")
