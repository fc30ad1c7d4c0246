"""The Fortran-subset translator (oracle/f90c.py) on small programs of this
project: gfortran semantics of the constructs RAM's kinetic step uses
(integer division, mixed-kind arithmetic, constant integer powers, array
sections and reductions, DO trip counts, SELECT CASE on blank-padded
strings, DATA/SAVE, derived types), stubs for untranslated calls, and a
loud failure for a reached statement outside the subset.

CPU only (gcc); no reference sources needed.
"""
import math
import subprocess

import numpy as np
import pytest

import f90c
import refrun

SRC = r"""
module TMod
  implicit none
  integer, parameter :: DP = kind(1.d0)
  integer :: n = 5, iq, ir, im, itrip, ilast, isel
  real(DP) :: x = 1.7, p2, p3, p4, p5, pr, rdiv, rmix, rmin, rmax, rsum, rneg
  real(DP), allocatable :: a(:), b(:,:)
  character(len=8) :: nm = 'He'
  logical :: lflag
  type Pair
     integer :: k
     real(DP) :: w
     character(len=4) :: tag
  end type Pair
  type(Pair), allocatable :: prs(:)
contains
  subroutine arith
    iq = -7/2
    ir = mod(-7, 2)
    rdiv = 1/2
    rmix = 1/2.
    p2 = x**2
    p3 = x**3
    p4 = x**4
    p5 = x**5
    pr = 10.**x
    rneg = -x**2
    im = 2**3*3
  end subroutine arith
  subroutine arrays
    integer :: i, j
    if (allocated(a)) deallocate(a)
    allocate(a(0:n), b(n, 3))
    a = 0.0
    do i = 0, n
       a(i) = i*1.5
    end do
    do j = 1, 3
       b(:, j) = a(1:n)*j
    end do
    b(2:3, 2) = -1.0
    rmin = minval(b)
    rmax = maxval(a)
    rsum = sum(b(:, 3))
  end subroutine arrays
  subroutine loops
    integer :: i, k
    itrip = 0
    do i = 5, 1
       itrip = itrip + 100
    end do
    do k = 10, 1, -3
       itrip = itrip + 1
    end do
    ilast = k
  end subroutine loops
  subroutine sel(code)
    integer, intent(in) :: code
    select case (nm)
    case ("H")
       isel = 1
    case ("He", "O")
       isel = 2
    case default
       isel = 3
    end select
    select case (code)
    case (1:3)
       isel = isel + 10
    case (7)
       isel = isel + 70
    end select
    lflag = trim(nm) == 'He' .and. .not. (nm /= 'He      ')
  end subroutine sel
  subroutine saved(k)
    integer, intent(inout) :: k
    integer :: tbl(3), cnt
    save cnt
    DATA tbl/4, 5, 6/
    cnt = cnt + 1
    k = tbl(k) * 10 + cnt
  end subroutine saved
  subroutine types
    if (allocated(prs)) deallocate(prs)
    allocate(prs(2))
    prs(1)%k = 3
    prs(1)%w = 2.5
    prs(1)%tag = 'ab'
    prs(2) = prs(1)
    prs(2)%k = 4
    iq = prs(2)%k + prs(1)%k
    x = prs(2)%w
    lflag = prs(2)%tag == 'ab'
  end subroutine types
  subroutine stubs_and_fail(k)
    integer, intent(in) :: k
    call not_translated(k)
    if (k > 0) then
       nm = 'a' // 'b'
    end if
  end subroutine stubs_and_fail
end module TMod
"""


@pytest.fixture(scope="module")
def tlib(tmp_path_factory):
    d = tmp_path_factory.mktemp("f90c")
    src = d / "tmod.f90"
    src.write_text(SRC)
    cpath, tr = f90c.translate_files([src], ["arith", "arrays", "loops", "sel", "saved", "types", "stubs_and_fail"],
                                     d, stem="tmod")
    lib = d / "libtmod.so"
    f90c.compile_c(cpath, lib, check=True)
    return refrun.RefLib.open(lib)


def test_integer_and_mixed_arithmetic(tlib):
    tlib.call("arith")
    assert tlib.get("tmod::iq") == -3 and tlib.get("tmod::ir") == -1
    assert tlib.get("tmod::rdiv") == 0.0 and tlib.get("tmod::rmix") == 0.5
    assert tlib.get("tmod::im") == 24
    x = 1.7
    assert tlib.get("tmod::p2") == x * x
    assert tlib.get("tmod::p3") == x * (x * x)
    assert tlib.get("tmod::p4") == (x * x) * (x * x)
    assert tlib.get("tmod::p5") == (x * (x * x)) * (x * x)
    assert tlib.get("tmod::pr") == math.pow(10.0, x)
    assert tlib.get("tmod::rneg") == -(x * x)


def test_sections_and_reductions(tlib):
    tlib.call("arrays")
    a = tlib.view("tmod::a")
    b = tlib.view("tmod::b")
    assert a.shape == (6,) and np.array_equal(a, np.arange(6) * 1.5)
    ref = np.stack([np.arange(1, 6) * 1.5 * j for j in (1, 2, 3)], axis=1)
    ref[1:3, 1] = -1.0
    assert np.array_equal(b, ref)
    assert tlib.get("tmod::rmin") == -1.0 and tlib.get("tmod::rmax") == 7.5
    assert tlib.get("tmod::rsum") == float(np.sum(ref[:, 2]))


def test_do_trip_counts(tlib):
    tlib.call("loops")
    assert tlib.get("tmod::itrip") == 4      # zero-trip loop, then 10,7,4,1
    assert tlib.get("tmod::ilast") == -2     # the DO variable after the last trip


def test_select_case_blank_padding(tlib):
    tlib.call("sel", 2)
    assert tlib.get("tmod::isel") == 12 and tlib.get("tmod::lflag") == 1
    tlib.call("sel", 7)
    assert tlib.get("tmod::isel") == 72
    tlib.call("sel", 5)
    assert tlib.get("tmod::isel") == 2


def test_data_and_save(tlib):
    assert tlib.call("saved", 2)[0] == 51
    assert tlib.call("saved", 3)[0] == 62


def test_derived_types(tlib):
    tlib.call("types")
    assert tlib.get("tmod::iq") == 7 and tlib.get("tmod::x") == 2.5 and tlib.get("tmod::lflag") == 1


def test_stub_counted_and_reached_failure_loud(tlib):
    tlib.lib.ref_stub_reset()
    rc, msg = tlib.call_rc("stubs_and_fail", 0)
    assert rc == 0 and tlib.stubs() == {"not_translated": 1}
    rc, msg = tlib.call_rc("stubs_and_fail", 1)
    assert rc == -1 and "concatenation" in msg and "tmod.f90" in msg


def test_bounds_checked_build_catches_out_of_range(tmp_path):
    src = tmp_path / "oob.f90"
    src.write_text("module Oob\n  real :: v(3)\ncontains\n  subroutine poke(i)\n    integer, intent(in) :: i\n"
                   "    v(i) = 1.0\n  end subroutine poke\nend module Oob\n")
    cpath, _ = f90c.translate_files([src], ["poke"], tmp_path, stem="oob")
    lib = tmp_path / "liboob.so"
    f90c.compile_c(cpath, lib, check=True)
    t = refrun.RefLib.open(lib)
    assert t.call_rc("poke", 3)[0] == 0
    rc, msg = t.call_rc("poke", 4)
    assert rc == -1 and "outside [1,3]" in msg
