"""Integer fixed-point log/exp of the transport kernel, compiled for the
host from the same header, against quad-precision references (correct
rounding) and the host libm (what the upstream CPU code calls)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_lib = None


def shim():
    global _lib
    if _lib is None:
        out_dir = os.path.join(ROOT, "branson_gb300", "_build")  # git-ignored build folder
        os.makedirs(out_dir, exist_ok=True)
        out = os.path.join(out_dir, "fixshim.so")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
               "-I", os.path.join(ROOT, "branson_gb300", "csrc"),
               os.path.join(ROOT, "tests", "fixmath_shim.cc"), "-o", out, "-lquadmath"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            pytest.skip("host quad-precision library unavailable: " + r.stderr[-200:])
        L = C.CDLL(out)
        for n in ("fix_neg_log_u53", "quad_neg_log_u53", "libm_neg_log_u53"):
            getattr(L, n).restype = C.c_double
            getattr(L, n).argtypes = [C.c_uint64]
        for n in ("fix_exp_neg", "quad_exp_neg", "libm_exp_neg"):
            getattr(L, n).restype = C.c_double
            getattr(L, n).argtypes = [C.c_double]
        _lib = L
    return _lib


def ulps(a, b):
    a, b = np.asarray(a), np.asarray(b)
    ia = a.view(np.int64)
    ib = b.view(np.int64)
    return np.abs(ia - ib)


def _mantissas(n, seed):
    rng = np.random.default_rng(seed)
    w = rng.integers(0, 2 ** 63, size=n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, size=n, dtype=np.uint64)
    m = (w >> np.uint64(11)) | np.uint64(1)
    edges = np.array([1, 3, 2 ** 52 - 1, 2 ** 52 + 1, 2 ** 53 - 1, 2 ** 53 - 3, 2 ** 53 - 2 ** 42 - 1,
                      2 ** 53 - 2 ** 42 + 1, 2 ** 52 + 2 ** 41 + 1, 3 * 2 ** 50 + 1], dtype=np.uint64)
    return np.concatenate([edges, m])


def test_neg_log_correctly_rounded():
    L = shim()
    ms = _mantissas(200000, 1)
    fix = np.array([L.fix_neg_log_u53(int(m)) for m in ms])
    ref = np.array([L.quad_neg_log_u53(int(m)) for m in ms])
    d = ulps(fix, ref)
    assert d.max() <= 1, f"max {d.max()} ulp"
    assert (d != 0).mean() < 2e-3, f"misrounded fraction {(d != 0).mean()}"
    libm = np.array([L.libm_neg_log_u53(int(m)) for m in ms])
    assert (fix == libm).mean() > 0.99


def test_neg_log_near_one():
    """u = 1 - n 2^-53 for small n takes the series branch."""
    L = shim()
    ms = np.uint64(2 ** 53) - np.arange(1, 5000, 2, dtype=np.uint64) * np.uint64(997)
    fix = np.array([L.fix_neg_log_u53(int(m)) for m in ms])
    ref = np.array([L.quad_neg_log_u53(int(m)) for m in ms])
    assert ulps(fix, ref).max() <= 1


def test_exp_neg_correctly_rounded():
    L = shim()
    rng = np.random.default_rng(2)
    taus = np.concatenate([rng.exponential(1.0, 100000), 10.0 ** rng.uniform(-18, 2.8, 100000),
                           [0.0, 5e-324, 1e-300, 2.0 ** -54, 2.0 ** -53, 1e-17, 0.5, 1.0, 700.0, 699.9]])
    fix = np.array([L.fix_exp_neg(float(t)) for t in taus])
    ref = np.array([L.quad_exp_neg(float(t)) for t in taus])
    d = ulps(fix, ref)
    assert d.max() <= 1, f"max {d.max()} ulp at tau={taus[np.argmax(d)]!r}"
    assert (d != 0).mean() < 2e-3
    libm = np.array([L.libm_exp_neg(float(t)) for t in taus])
    assert (fix == libm).mean() > 0.99


def _sincos(L, name, phis):
    fn = getattr(L, name)
    fn.argtypes = [C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    s, c = C.c_double(), C.c_double()
    out = np.empty((len(phis), 2))
    for i, p in enumerate(phis):
        fn(float(p), C.byref(s), C.byref(c))
        out[i] = (s.value, c.value)
    return out


def test_sincos_correctly_rounded():
    """phi = (2u)*pi as the upstream sampler forms it, plus the doubles next
    to multiples of pi/2 where one result is tiny."""
    L = shim()
    ms = _mantissas(100000, 3)
    u = ms.astype(np.float64) * 2.0 ** -53
    phis = u * 2.0 * np.pi
    near = []
    for k in (1, 2, 3):
        x = k * np.pi / 2
        for d in range(-3, 4):
            near.append(np.nextafter(x, 10.0) if d > 0 else x)
            x = np.nextafter(x, 10.0 if d > 0 else 0.0)
    phis = np.concatenate([phis, near, [1e-15, 2.0 ** -40, 6.283185307179586]])
    fix = _sincos(L, "fix_sincos", phis)
    ref = _sincos(L, "quad_sincos", phis)
    d = ulps(fix.ravel(), ref.ravel())
    assert d.max() <= 1, f"max {d.max()} ulp at {phis[np.argmax(d) // 2]!r}"
    assert (d != 0).mean() < 2e-3, (d != 0).mean()
    libm = _sincos(L, "libm_sincos", phis)
    assert (fix.ravel() == libm.ravel()).mean() > 0.99


def _bind_exact(L):
    L.fix_sqrt.restype = C.c_double
    L.fix_sqrt.argtypes = [C.c_double]


def test_sqrt_matches_ieee_bitwise():
    L = shim()
    _bind_exact(L)
    rng = np.random.default_rng(6)
    x = np.concatenate([rng.uniform(0, 1, 100000) ** 3, 10.0 ** rng.uniform(-300, 300, 20000),
                        [1.0, 0.25, np.nextafter(1.0, 0), 2.0 ** -51, 3.0, 4.0, np.nextafter(4.0, 0)]])
    got = np.array([L.fix_sqrt(v) for v in x])
    assert np.array_equal(got.view(np.int64), np.sqrt(x).view(np.int64))


def test_division_by_stored_reciprocal_is_ieee(tmp_path):
    """The transport kernels divide by a stored reciprocal with two fma
    (Markstein's final step); the quotient must be the IEEE one bit for bit."""
    import shutil
    import subprocess
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not available")
    src = os.path.join(os.path.dirname(__file__), "div_recip_check.c")
    exe = str(tmp_path / "div_recip_check")
    subprocess.run([cc, "-O2", "-std=c11", "-ffp-contract=off", "-o", exe, src, "-lm"], check=True)
    r = subprocess.run([exe, "3000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
