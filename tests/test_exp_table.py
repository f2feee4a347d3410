"""The table-driven exponential of the rate code (`tab_exp`, spitfire_gb300/csrc/chem_device.cuh): the committed
constants are what their generator writes, and the method's arithmetic, restated on the host operation for operation
(every FMA rounded once, through exact rationals), reproduces e^x to within 0.52 ulp against a 300-bit reference,
for arguments across the whole normal range and the thermodynamic one."""
import importlib.util
import os
import re
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, 'spitfire_gb300', 'csrc')


def _gen():
    spec = importlib.util.spec_from_file_location('gen_exp_table', os.path.join(CSRC, 'gen_exp_table.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _constants():
    text = open(os.path.join(CSRC, 'exp_table.h')).read()
    val = lambda name: float.fromhex(re.search(name + r' = (\S+);', text).group(1))
    body = text[text.index('kExpTable[128] = {') + len('kExpTable[128] = {'):text.index('};')]
    tab = [float.fromhex(v) for v in body.replace('\n', ' ').split(',') if v.strip()]
    return val('kExpInvL'), val('kExpL1'), val('kExpL2'), tab


def _fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _tab_exp(x, inv_l, l1, l2, tab):
    """tab_exp's operations in order (the normal-result path, |x| < 708)."""
    magic = 1.5 * 2. ** 52
    tm = _fma(x, inv_l, magic)
    n = int(tm - magic)
    nd = tm - magic
    r = _fma(-nd, l2, _fma(-nd, l1, x))
    q = _fma(r, 1. / 720., 1. / 120.)
    q = _fma(r, q, 1. / 24.)
    q = _fma(r, q, 1. / 6.)
    q = _fma(r, q, 0.5)
    p = _fma(q, r * r, r)
    j, m = n & 63, n >> 6
    y = tab[2 * j] + _fma(tab[2 * j], p, tab[2 * j + 1])
    return float(np.ldexp(y, m))


def test_header_is_what_the_generator_writes():
    pytest.importorskip('mpmath')
    assert _gen().header_text() == open(os.path.join(CSRC, 'exp_table.h')).read()


def test_method_reproduces_exp_within_half_an_ulp_and_a_bit():
    mp = pytest.importorskip('mpmath')
    mp.mp.prec = 300
    inv_l, l1, l2, tab = _constants()
    assert len(tab) == 128
    for j in range(64):  # head + tail = 2^(j/64) to far below an ulp of the head
        err = abs(mp.mpf(tab[2 * j]) + mp.mpf(tab[2 * j + 1]) - mp.power(2, mp.mpf(j) / 64))
        assert err < mp.mpf(2) ** -100
    rng = np.random.default_rng(5)
    xs = np.concatenate([rng.uniform(-707.9, 707.9, 400), rng.uniform(-80., 5., 400), rng.uniform(-0.02, 0.02, 200),
                         [0., -0., 1., -1., 1e-300, 707.9, -707.9, np.log(2.) / 128, -np.log(2.) / 128]])
    worst = 0.
    for x in xs:
        v = _tab_exp(float(x), inv_l, l1, l2, tab)
        ref = mp.exp(mp.mpf(float(x)))
        ulp = np.spacing(float(ref))
        worst = max(worst, float(abs(mp.mpf(v) - ref) / ulp))
    assert worst < 0.52, worst
