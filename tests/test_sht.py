"""Spin-weighted transforms: the oracle pinned to closed forms and to the
reference's own properties (tests/TestSpinMachinery.cpp:33-165: round trip to
1e-12 for N = -2..2, reality relations), then the GPU grid against the oracle."""

import math
from fractions import Fraction

import numpy as np
import pytest
import scipy.special as sp

from tests import _oracle


def noise(k):
    """The reference tests' deterministic stream in [-1, 1)."""
    v = math.sin(12.9898 * (k + 1)) * 43758.5453
    return v - math.floor(v) - 0.5


def edmonds_d(l, mp, m, beta):
    """Wigner d^l_{m'm}(beta), Edmonds' convention, exact factorial sum."""
    total = 0.0
    f = math.factorial
    pref = math.sqrt(f(l + mp) * f(l - mp) * f(l + m) * f(l - m))
    for k in range(0, 2 * l + 1):
        a, b, c, d = l + m - k, k, l - k - mp, k - m + mp
        if min(a, b, c, d) < 0:
            continue
        sign = -1.0 if (k - m + mp) % 2 else 1.0
        total += sign * pref / (f(a) * f(b) * f(c) * f(d)) * \
            math.cos(beta / 2) ** (2 * l - 2 * k + m - mp) * math.sin(beta / 2) ** (2 * k - m + mp)
    return total


def test_gauss_legendre_integrates_polynomials():
    x, w = _oracle.gauss_legendre(17)
    assert np.all(np.diff(x) < 0)  # increasing colatitude
    for k in range(0, 34):
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs(np.sum(w * x ** k) - exact) < 1e-14


@pytest.mark.parametrize("N", [-2, -1, 0, 1, 2])
def test_wigner_table_matches_the_exact_sum(N):
    lmax = 12
    theta = np.array([0.13, 0.7, 1.3, 2.2, 3.0])
    for m in range(-lmax, lmax + 1):
        table = _oracle.wigner_column(lmax, N, m, theta)
        l0 = max(abs(m), abs(N))
        for l in range(l0, lmax + 1):
            for j, t in enumerate(theta):
                # d^l_{Nm} of the basis is Edmonds' d^l_{mN}
                want = math.sqrt((2 * l + 1) / (4 * math.pi)) * edmonds_d(l, m, N, t)
                assert abs(table[l - l0, j] - want) < 1e-13, (N, m, l, t)


def test_spin_zero_is_the_condon_shortley_harmonic():
    lmax = 20
    theta = np.array([0.05, 0.9, 1.7, 2.9])
    for m in range(0, lmax + 1):
        table = _oracle.wigner_column(lmax, 0, m, theta)
        for l in range(m, lmax + 1):
            want = sp.sph_harm_y(l, m, theta, 0.0).real
            assert np.max(np.abs(table[l - m] - want)) < 1e-13


def test_wigner_table_is_orthonormal_at_lmax_256():
    lmax = 256
    theta, w, _ = _oracle.grid(lmax, 1.5)
    for N in (-2, -1, 0):
        for m in (-256, -131, -2, -1, 0, 1, 7, 128, 255):
            if max(abs(m), abs(N)) > lmax:
                continue
            t = _oracle.wigner_column(lmax, N, m, theta)
            gram = (t * w) @ t.T * 2.0 * np.pi
            assert np.max(np.abs(gram - np.eye(gram.shape[0]))) < 1e-12, (N, m)


def random_spin_coefficients(lmax, N, salt=0):
    size = (lmax + 1) ** 2 - N * N
    out = np.zeros(size, dtype=np.complex128)
    for l in range(abs(N), lmax + 1):
        for m in range(-l, l + 1):
            k = l * l - N * N + m + l
            out[k] = complex(noise(7 * k + N + 2 + salt), noise(11 * k + salt))
    return out


def hermitian_real_coefficients(lmax, salt=0):
    out = np.zeros((lmax + 1) * (lmax + 2) // 2, dtype=np.complex128)
    for l in range(lmax + 1):
        for m in range(l + 1):
            k = l * (l + 1) // 2 + m
            out[k] = complex(noise(5 * k + salt), 0.0 if m == 0 else noise(13 * k + salt))
    return out


@pytest.mark.parametrize("N", [-2, -1, 0, 1, 2])
def test_oracle_spin_round_trip(N):
    lmax = 12
    theta, w, nphi = _oracle.grid(lmax, 1.0)
    c = random_spin_coefficients(lmax, N)
    f = _oracle.synthesise_spin(lmax, N, theta, nphi, c)
    back = _oracle.expand_spin(lmax, N, theta, w, nphi, f)
    assert np.max(np.abs(back - c)) < 1e-12 * np.max(np.abs(c))


def test_oracle_real_round_trip_and_complex_agreement():
    lmax = 12
    theta, w, nphi = _oracle.grid(lmax, 1.5)
    c = hermitian_real_coefficients(lmax)
    f = _oracle.synthesise_real(lmax, theta, nphi, c)
    back = _oracle.expand_real(lmax, theta, w, nphi, f)
    assert np.max(np.abs(back - c)) < 1e-12
    # the same field through the complex spin-0 transform with the m < 0 twins
    full = np.zeros((lmax + 1) ** 2, dtype=np.complex128)
    for l in range(lmax + 1):
        for m in range(l + 1):
            v = c[l * (l + 1) // 2 + m]
            full[l * l + m + l] = v
            full[l * l - m + l] = (-1) ** m * np.conj(v)
    fc = _oracle.synthesise_spin(lmax, 0, theta, nphi, full)
    assert np.max(np.abs(fc.imag)) < 1e-12
    assert np.max(np.abs(fc.real - f)) < 1e-12


def test_oracle_reality_relation_of_the_basis():
    # conj(Y^N_lm) = (-1)^(N - m) Y^(-N)_(l,-m) (tests/TestSpinMachinery.cpp:110-165)
    lmax = 8
    theta, w, nphi = _oracle.grid(lmax, 1.0)
    for N in (1, 2):
        for l in range(N, lmax + 1):
            for m in range(-l, l + 1):
                a = np.zeros((lmax + 1) ** 2 - N * N, dtype=np.complex128)
                a[l * l - N * N + m + l] = 1.0
                b = np.zeros((lmax + 1) ** 2 - N * N, dtype=np.complex128)
                b[l * l - N * N - m + l] = (-1.0) ** (N - m)
                ya = _oracle.synthesise_spin(lmax, N, theta, nphi, a)
                yb = _oracle.synthesise_spin(lmax, -N, theta, nphi, b)
                assert np.max(np.abs(np.conj(ya) - yb)) < 1e-13


# -- the GPU grid --------------------------------------------------------------------------

def _grid_and_oracle_grid(lmax, oversampling, nmax=2, fp64_emulation=False):
    from sl3dpp_gb300.grid import SurfaceGrid

    g = SurfaceGrid(lmax, nmax, oversampling, fp64_emulation)
    theta, w, nphi = _oracle.grid(lmax, oversampling)
    assert g.ntheta == theta.size and g.nphi == nphi
    assert np.max(np.abs(g.theta - theta)) < 1e-15
    assert np.max(np.abs(g.weights - w)) < 1e-15
    return g, theta, w, nphi


@pytest.mark.gpu
@pytest.mark.parametrize("emulated", [False, True])
@pytest.mark.parametrize("lmax,oversampling,count", [(12, 1.0, 1), (12, 1.0, 3), (16, 1.5, 5), (33, 1.5, 2),
                                                     (20, 1.0, 9)])
def test_gpu_spin_transforms_match_oracle(gpu, lmax, oversampling, count, emulated):
    """Both forms of the FP64 contraction, the FP64 units' and the tensor
    cores' emulation, at the FP64 bar (1e-12 of the largest value). Counts 1
    to 8 (2 to 16 columns) take the FP64 units' few-column kernels, 9 the
    tiled one."""
    import torch

    g, theta, w, nphi = _grid_and_oracle_grid(lmax, oversampling, fp64_emulation=emulated)
    for N in (-2, -1, 0, 1, 2):
        cs = [random_spin_coefficients(lmax, N, salt=17 * p) for p in range(count)]
        want = np.concatenate([_oracle.synthesise_spin(lmax, N, theta, nphi, c) for c in cs])
        got = g.SynthesiseSpinBatch(N, torch.tensor(np.concatenate(cs), device=gpu), count).cpu().numpy()
        assert np.max(np.abs(got - want)) < 1e-12 * np.max(np.abs(want)), N
        back_want = np.concatenate([_oracle.expand_spin(lmax, N, theta, w, nphi, want[p * g.FieldSize():(p + 1) * g.FieldSize()])
                                    for p in range(count)])
        back = g.ExpandSpinBatch(N, torch.tensor(want, device=gpu), count).cpu().numpy()
        assert np.max(np.abs(back - back_want)) < 1e-12 * np.max(np.abs(back_want)), N
        assert np.max(np.abs(back - np.concatenate(cs))) < 1e-12 * np.max(np.abs(np.concatenate(cs)))


@pytest.mark.gpu
@pytest.mark.parametrize("emulated", [False, True])
@pytest.mark.parametrize("lmax,oversampling,count", [(12, 1.0, 1), (12, 1.0, 3), (32, 1.5, 4), (24, 1.5, 8),
                                                     (20, 1.0, 9)])
def test_gpu_real_transforms_match_oracle(gpu, lmax, oversampling, count, emulated):
    import torch

    g, theta, w, nphi = _grid_and_oracle_grid(lmax, oversampling, fp64_emulation=emulated)
    cs = [hermitian_real_coefficients(lmax, salt=3 * p) for p in range(count)]
    want = np.concatenate([_oracle.synthesise_real(lmax, theta, nphi, c) for c in cs])
    got = g.SynthesiseBatch(torch.tensor(np.concatenate(cs), device=gpu), count).cpu().numpy()
    assert np.max(np.abs(got - want)) < 1e-12 * np.max(np.abs(want))
    # a field that is not band-limited: W(x) times the synthesised one
    tt, pp = np.meshgrid(theta, np.arange(nphi) * 2 * np.pi / nphi, indexing="ij")
    weight = np.exp(0.5 * np.cos(tt) * np.sin(3 * pp)).ravel()
    fields = want * np.tile(weight, count)
    back_want = np.concatenate([_oracle.expand_real(lmax, theta, w, nphi, fields[p * g.FieldSize():(p + 1) * g.FieldSize()])
                                for p in range(count)])
    back = g.ExpandBatch(torch.tensor(fields, device=gpu), count).cpu().numpy()
    assert np.max(np.abs(back - back_want)) < 1e-12 * np.max(np.abs(back_want))


@pytest.mark.gpu
@pytest.mark.parametrize("emulated", [False, True])
def test_gpu_round_trip_at_lmax_256(gpu, emulated):
    import torch

    lmax = 256
    from sl3dpp_gb300.grid import SurfaceGrid

    g = SurfaceGrid(lmax, 2, 1.5, emulated)
    assert (g.ntheta, g.nphi) == (385, 800)
    rng = np.random.default_rng(5)
    for N in (-2, -1):
        size = g.SpinCoefficientSize(N)
        c = torch.tensor(rng.standard_normal(2 * size).view(np.complex128), device=gpu)
        back = g.ExpandSpinBatch(N, g.SynthesiseSpinBatch(N, c, 1), 1)
        assert (back - c).abs().max().item() < 1e-11 * c.abs().max().item()


@pytest.mark.gpu
def test_gpu_emulated_fp64_contraction_agrees_with_the_fp64_units(gpu):
    """The tensor-core emulation against the FP64 units on the same inputs at
    lmax 256 (depth 385 in the analysis, near the exactness bound): agreement
    to about 2^-45 of the largest value, both directions, coefficients whose
    magnitudes span ten decades."""
    import torch

    from sl3dpp_gb300.grid import SurfaceGrid

    lmax = 256
    native, emulated = SurfaceGrid(lmax, 2, 1.5), SurfaceGrid(lmax, 2, 1.5, True)
    rng = np.random.default_rng(9)
    for N in (-2, 0):
        size = native.SpinCoefficientSize(N)
        mag = 10.0 ** rng.uniform(-10, 0, size)
        c = torch.tensor((rng.standard_normal(2 * size).view(np.complex128)) * mag, device=gpu)
        fa, fb = native.SynthesiseSpinBatch(N, c, 1), emulated.SynthesiseSpinBatch(N, c, 1)
        assert (fa - fb).abs().max().item() < 3e-14 * fa.abs().max().item(), N
        ba, bb = native.ExpandSpinBatch(N, fa, 1), emulated.ExpandSpinBatch(N, fa, 1)
        assert (ba - bb).abs().max().item() < 3e-14 * ba.abs().max().item(), N


@pytest.mark.gpu
@pytest.mark.parametrize("lmax,count", [(33, 5), (64, 40), (64, 80)])
@pytest.mark.parametrize("N,real", [(-2, False), (-1, False), (0, True)])
def test_gpu_fp32_tensor_core_contraction_matches_fp64(gpu, lmax, count, N, real):
    """The 3xTF32 tensor-core contraction of the correction passes (FP32
    buffers) against the FP64 one on the same inputs, both directions, in the
    device layouts: within 4e-6 of the largest value. count 5 and 40 take the
    paired MMA (B's high and low parts in one operand, 2 x 16 and 2 x 80
    columns), count 80 (160 columns) the three separate products."""
    import torch

    from sl3dpp_gb300 import _lib
    from sl3dpp_gb300.grid import SurfaceGrid

    g = SurfaceGrid(lmax, 2, 1.5)
    lib = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    rows = g.CoefficientSize() if real else g.SpinCoefficientSize(N)
    mcount = lmax + 1 if real else 2 * lmax + 1
    rng = np.random.default_rng(100 * lmax + 7 * count - N)
    coeffs = torch.tensor(rng.standard_normal(rows * count * 2), device=gpu)
    spectra = torch.tensor(rng.standard_normal(mcount * g.ntheta * count * 2), device=gpu)
    for analysis, src, size in ((0, coeffs, mcount * g.ntheta * count * 2), (1, spectra, rows * count * 2)):
        out64 = torch.zeros(size, dtype=torch.float64, device=gpu)
        out32 = torch.zeros(size, dtype=torch.float32, device=gpu)
        src32 = src.float().contiguous()
        _lib.check(lib.sl3dgpu_legendre_device(g._handle, N, int(real), analysis, 0, src.data_ptr(), count,
                                               out64.data_ptr(), stream))
        _lib.check(lib.sl3dgpu_legendre_device(g._handle, N, int(real), analysis, 1, src32.data_ptr(), count,
                                               out32.data_ptr(), stream))
        torch.cuda.synchronize()
        # the FP64 contraction of the FP32-rounded input is the reference
        ref = torch.zeros(size, dtype=torch.float64, device=gpu)
        rounded = src32.double()
        _lib.check(lib.sl3dgpu_legendre_device(g._handle, N, int(real), analysis, 0, rounded.data_ptr(), count,
                                               ref.data_ptr(), stream))
        torch.cuda.synchronize()
        scale = ref.abs().max().item()
        assert scale > 0
        assert (out32.double() - ref).abs().max().item() < 4e-6 * scale, (analysis, N)
        assert (out64 - ref).abs().max().item() < 1e-6 * scale  # the rounding of the input only
