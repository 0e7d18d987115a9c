"""The functor surface of both front ends, checked without a GPU: the Python
aliases of boost.simd's float forms (inc, dec, abss, negs, sqrs, conj) lower
to the same run-time compiled kernel as the expressions they stand for, and a
C++ translation unit that calls the table layer's distribution, select,
quotient and exponent functors compiles against nt2/table.hpp."""
import os
import shutil
import subprocess

import pytest
import torch

from nt2_gb300 import expr as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _source(e):
    prog, _ = E.compile_program([torch.zeros(8)], [e])
    return prog.jit_source(0)


@pytest.mark.parametrize("alias,same", [
    ("inc", lambda x: x + 1.0), ("dec", lambda x: x - 1.0), ("abss", lambda x: E.abs_(x)),
    ("negs", lambda x: -x), ("sqrs", lambda x: E.sqr(x))])
def test_float_aliases_lower_like_their_definitions(alias, same):
    x = E.Table(torch.zeros(8))
    assert _source(getattr(E, alias)(x)) == _source(same(x))
    assert E.conj(x) is x  # the identity on reals


def test_cpp_functor_surface_compiles(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "surface.cpp"
    src.write_text("""#include <nt2/table.hpp>
int main()
{
    nt2::table<float, nt2::device_> a(nt2::of_size(8));
    auto e = nt2::inc(a) + nt2::dec(a) + nt2::abss(a) + nt2::negs(a) + nt2::sqrs(a) + nt2::maxnum(a, a) +
             nt2::minnum(a, 1.0f) + nt2::maxmag(a, a) + nt2::minmag(a, a) + nt2::minmod(a, a) + nt2::negate(a, a) +
             nt2::fms(a, a, 0.5f) + nt2::fnma(a, a, a) + nt2::divfloor(a, 2.0f) + nt2::divceil(a, a) +
             nt2::divfix(a, a) + nt2::divround(a, a) + nt2::divround2even(a, a) + nt2::mod(a, a) + nt2::rem(a, 3.0f) +
             nt2::pow2(a) + nt2::pow2(a, a) + nt2::proper_tanpi(a) + nt2::cauinv(a) + nt2::cauinv(a, 1.0f) +
             nt2::cauinv(a, 1.0f, 2.0f) + nt2::normpdf(a, 0.5f, 2.0f) + nt2::evinv(a, a, a);
    (void)e;
    return 0;
}
""")
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "nt2_gb300", "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[:2000]
