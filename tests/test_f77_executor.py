"""The Fortran 77 subset executor (oracle/f77.py) on small programs whose
results are known: the golden vectors it produces are only as good as its
semantics."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
import f77  # noqa: E402
from f77 import Ref  # noqa: E402

SRC = """\
c     fixed form: labels in 1-5, continuation in 6, code to column 72
      subroutine loops(n, s, t)
      integer n, s, t
      s = 0
      do 10 i = 1, n
      do 10 j = 1, i
         s = s + j
   10 continue
      t = 0
      do i = n, 1, -2
         t = t*10
     $       + i
      enddo
      return
      end
c-----------------------------------------------------------------------
      function isum(a, n)
      integer a(n)
      isum = 0
      do k = 1, n
         if (a(k) .lt. 0) goto 20
         isum = isum + a(k)
      enddo
   20 continue
      return
      end
c-----------------------------------------------------------------------
      subroutine arith(r)
      real r(8)
      integer i, j
      i = -7
      j = 2
      r(1) = i/j
      r(2) = mod(i, j)
      i = 65536
      r(3) = i*i
      r(4) = 2.**10
      r(5) = 3.0**3
      r(6) = 1.0/3.0
      r(7) = .5d0 + 1.e-1
      r(8) = sign(2.0, -1.0)
      return
      end
c-----------------------------------------------------------------------
      subroutine passthru(u, n)
      call fill(u, n)
      return
      end
      subroutine fill(v, n)
      real v(n)
      do i = 1, n
         v(i) = i
      enddo
      return
      end
c-----------------------------------------------------------------------
      subroutine shifted(a)
      real a(-1:3, 2)
      a(-1, 1) = 10.
      a(3, 2) = 20.
      return
      end
c-----------------------------------------------------------------------
      subroutine blocks(k, r)
      integer k
      real r
      if (k .eq. 1) then
         r = 1.
      else if (k .eq. 2) then
         r = 2.
      else
         r = 3.
      endif
      if (k .gt. 5) r = -r
      return
      end
c-----------------------------------------------------------------------
      subroutine backjump(n, m)
      integer n, m
      m = 0
   30 m = m + 1
      if (m .lt. n) goto 30
      return
      end
c-----------------------------------------------------------------------
      subroutine comm(v)
      common /blk/ a, ib(3)
      integer ib
      a = v
      ib(2) = 5
      return
      end
c-----------------------------------------------------------------------
      subroutine datasv(k)
      integer kk
      data kk /41/
      save kk
      kk = kk + 1
      k = kk
      return
      end
c-----------------------------------------------------------------------
      subroutine autoarr(n, s)
      common /dims/ m
      real w(m, n)
      s = 0.
      do j = 1, n
         do i = 1, m
            w(i, j) = i + 10*j
            s = s + w(i, j)
         enddo
      enddo
      return
      end
"""


@pytest.fixture(scope="module")
def rt(tmp_path_factory):
    p = tmp_path_factory.mktemp("f77") / "t.f"
    p.write_text(SRC)
    return f77.F77([str(p)], [str(p.parent)])


def test_loops_shared_terminal_and_negative_step(rt):
    s, t = [0], [0]
    rt.call("loops", 5, s, t)
    assert s[0] == sum(j for i in range(1, 6) for j in range(1, i + 1))
    assert t[0] == 531


def test_function_goto_out_of_loop(rt):
    assert rt.call("isum", [3, 4, -1, 100], 4) == 7
    assert rt.call("isum", [3, 4, 1, 100], 4) == 108


def test_integer_and_real_semantics(rt):
    r = [0.0] * 8
    rt.call("arith", r)
    assert r[0] == -3.0            # truncation toward zero
    assert r[1] == -1.0            # mod takes the dividend's sign
    assert r[2] == 0.0             # 65536*65536 wraps in 32 bits
    assert r[3] == 1024.0
    assert r[4] == 27.0
    assert r[5] == 1.0 / 3.0       # default REAL is double
    assert r[6] == 0.5 + 0.1
    assert r[7] == -2.0


def test_undeclared_dummy_passes_the_array_through(rt):
    u = [0.0] * 4
    rt.call("passthru", u, 4)
    assert u == [1.0, 2.0, 3.0, 4.0]


def test_lower_bounds_column_major(rt):
    a = [0.0] * 10
    rt.call("shifted", a)
    assert a[0] == 10.0 and a[9] == 20.0


def test_block_and_logical_if(rt):
    out = []
    for k in (1, 2, 3, 7):
        r = [0.0]
        rt.call("blocks", k, r)
        out.append(r[0])
    assert out == [1.0, 2.0, 3.0, -3.0]


def test_backward_goto(rt):
    m = [0]
    rt.call("backjump", 4, m)
    assert m[0] == 4


def test_common_blocks_shared_storage(rt):
    rt.call("comm", 2.5)
    blk = rt.common("blk")
    assert blk[0][0] == 2.5 and blk[1] == [0, 5, 0]


def test_data_and_save_persist(rt):
    k = [0]
    rt.call("datasv", k)
    rt.call("datasv", k)
    assert k[0] == 43


def test_automatic_array(rt):
    rt.ensure_common("dims")[0][0] = 3
    s = [0.0]
    rt.call("autoarr", 2, s)
    assert s[0] == sum(i + 10 * j for i in range(1, 4) for j in range(1, 3))


def test_unknown_routine_is_an_error(tmp_path):
    p = tmp_path / "u.f"
    p.write_text("      subroutine a()\n      call nothere()\n      return\n      end\n")
    r = f77.F77([str(p)], [str(tmp_path)])
    with pytest.raises(f77.F77Error):
        r.call("a")
