"""The design filters with a general weight functor on the GPU.

HeavisideFilter::GetFilteredVariable / GetFilteredSensitivity (heavisidefilter.h:404-899) and
DensityFilter::GetFilteredValue (densityfilter.h:10-515) take a weight functor
`_weight(i1, j1, k1, i2, j2, k2)` evaluated for every node and every tap within R (taps outside
the lattice skipped). The restatement below follows those loops: per node, taps in the (i2, j2,
k2) loop order, sum of weight * value and of weight; the Heaviside projection
0.5 (tanh(beta/2) + tanh(beta (x - 1/2))) / tanh(beta/2) of the average; the sensitivity as
dfdrho * dH/dx at each node, then averaged with the same weights. Checked through the C ABI
(`pl_filter_weighted` with a random weight table) and through the drop-in template API
(tests/dropin/filter_driver.cpp: the default hat, a hat on a design region, a Gaussian), FP64,
to 1e-12."""
import math
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "panslbm2_gb300")


def taps(nd, R):
    nR, out = int(R), []
    for a in range(-nR, nR + 1):
        for b in range(-nR, nR + 1):
            for c in (range(-nR, nR + 1) if nd == 3 else [0]):
                d = math.sqrt(a * a + b * b + c * c)
                if d <= R:
                    out.append((a, b, c))
    return out


def grid(shape):
    nx, ny, nz = shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return i.ravel(), j.ravel(), k.ravel()


def average(nd, shape, R, v, wfun):
    nx, ny, nz = shape
    i, j, k = grid(shape)
    ws, w = np.zeros(i.size), np.zeros(i.size)
    for t, (a, b, c) in enumerate(taps(nd, R)):
        i2, j2, k2 = i + a, j + b, k + c
        ok = (i2 >= 0) & (i2 < nx) & (j2 >= 0) & (j2 < ny) & (k2 >= 0) & (k2 < nz)
        wt = wfun(t, i, j, k, i2, j2, k2)
        id2 = i2 + nx * (j2 + ny * k2)
        ws[ok] += wt[ok] * v[id2[ok]]
        w[ok] += wt[ok]
    return ws / w


def heaviside(x, beta):
    return 0.5 * (math.tanh(0.5 * beta) + np.tanh(beta * (x - 0.5))) / math.tanh(0.5 * beta)


def filters(nd, shape, R, beta, s, d, wfun):
    x = average(nd, shape, R, s, wfun)
    th = np.tanh(beta * (x - 0.5))
    tmp = d * (0.5 * beta * (1.0 - th * th) / math.tanh(0.5 * beta))
    return heaviside(x, beta), average(nd, shape, R, tmp, wfun), x


def close(a, b, tol=1e-12):
    err = float(np.max(np.abs(a - b)) / max(1e-300, float(np.max(np.abs(b)))))
    assert err <= tol, "max rel err %.3e" % err


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("nd,shape,R", [(2, (40, 30, 1), 3.0), (3, (14, 12, 10), 2.5)])
def test_capi_weight_table(torch_cuda, nd, shape, R):
    from panslbm2_gb300.lattice import LatticePair
    q = 9 if nd == 2 else 15
    lp = LatticePair(q, *shape, "fp64")
    try:
        n = shape[0] * shape[1] * shape[2]
        rng = np.random.default_rng(3)
        s, d = rng.random(n), rng.standard_normal(n)
        di, dj, dk = lp.filter_taps(R)
        tp = taps(nd, R)
        assert list(zip(di.tolist(), dj.tolist(), dk.tolist())) == tp
        table = 0.1 + rng.random((n, len(tp)))
        wfun = lambda t, i, j, k, i2, j2, k2: table[i + shape[0] * (j + shape[1] * k), t]  # noqa: E731
        ref_v, ref_s, ref_a = filters(nd, shape, R, 8.0, s, d, wfun)
        close(lp.filter_weighted(0, R, s, table, beta=8.0), ref_v)
        close(lp.filter_weighted(1, R, s, table, b=d, beta=8.0), ref_s)
        close(lp.filter_weighted(2, R, s, table), ref_a)
        # the hat weights as a table give the library's own hat filter
        hat = np.array([(R - math.sqrt(a * a + b * b + c * c)) / R for (a, b, c) in tp])
        close(lp.filter_weighted(0, R, s, np.tile(hat, (n, 1)), beta=8.0), lp.heaviside_var(R, 8.0, s))
    finally:
        lp.close()


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    out = str(tmp_path_factory.mktemp("dropin") / "filter_driver")
    subprocess.check_call([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "dropin", "filter_driver.cpp"), "-L", LIBDIR,
                           "-lpanslbm_gb300", "-Wl,-rpath," + LIBDIR, "-o", out])
    return out


@pytest.mark.parametrize("nd,shape,R", [(2, (40, 30, 1), 3.0), (3, (14, 12, 10), 2.5)])
def test_dropin_weight_functors(torch_cuda, driver, tmp_path, nd, shape, R):
    n = shape[0] * shape[1] * shape[2]
    beta = 8.0
    rng = np.random.default_rng(11)
    s, d = rng.random(n), rng.standard_normal(n)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as fh:
        fh.write(struct.pack("4i", nd, *shape))
        fh.write(struct.pack("2d", R, beta))
        fh.write(s.tobytes())
        fh.write(d.tobytes())
    subprocess.check_call([driver, str(fin), str(fout)])
    got = np.fromfile(fout, np.float64).reshape(3, 3, n)
    tp = taps(nd, R)
    dist = [math.sqrt(a * a + b * b + c * c) for (a, b, c) in tp]
    half = shape[1] // 2

    def hat(t, i, j, k, i2, j2, k2):
        return np.full(i.size, (R - dist[t]) / R)

    def region(t, i, j, k, i2, j2, k2):
        both = (j < half) & (j2 < half)
        return np.where(both, (R - dist[t]) / R, 1.0 if dist[t] == 0.0 else 0.0)

    def gauss(t, i, j, k, i2, j2, k2):
        return np.exp(-((i - i2) ** 2.0 + (j - j2) ** 2.0 + (k - k2) ** 2.0) / R)

    for m, wfun in enumerate((hat, region, gauss)):
        ref = filters(nd, shape, R, beta, s, d, wfun)
        for o in range(3):
            close(got[m, o], ref[o])
