"""The overlap schedule's ticket order (csrc/vox_schedule.h) on the host: every generation
and emission item appears exactly once, the tickets past the items are the end markers,
and the chunk of every emission item, with every chunk before it, has a smaller ticket
than the item. The last property is what makes every device-side wait of the overlap
kernel end without co-residency: an item waits only for items with smaller tickets, which
running CTAs hold or have finished."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(REPO, "wgpu-voxel-engine_gb300", "csrc")

CHECK = r"""
#include <cstdio>
#include <vector>
#include "vox_schedule.h"

static int check(unsigned n, unsigned split, unsigned lag, unsigned grid) {
  const unsigned items = n * split;
  const unsigned L = lag > n ? n : lag;  // the kernel clamps the lag the same way
  std::vector<long> a_ticket(n, -1), c_ticket(items, -1);
  for (unsigned t = 0; t < n + items + grid; ++t) {
    unsigned idx = 0;
    const int kind = vox::overlap_ticket(t, n, items, L, idx);
    if (t >= n + items) {
      if (kind != 2) return 1;  // past the items: end markers only
      continue;
    }
    if (kind == 0) {
      if (idx >= n || a_ticket[idx] >= 0) return 2;
      a_ticket[idx] = t;
    } else if (kind == 1) {
      if (idx >= items || c_ticket[idx] >= 0) return 3;
      c_ticket[idx] = t;
    } else {
      return 4;  // an end marker before the last item
    }
  }
  long highest_a = -1;  // highest generation ticket among chunks 0..c
  unsigned c_seen = 0;
  for (unsigned m = 0; m < items; ++m) {
    if (c_ticket[m] < 0) return 5;
    const unsigned c = m / split;
    for (; c_seen <= c; ++c_seen) {
      if (a_ticket[c_seen] < 0) return 6;
      if (a_ticket[c_seen] > highest_a) highest_a = a_ticket[c_seen];
    }
    if (highest_a >= c_ticket[m]) return 7;  // waits for a later ticket
  }
  return 0;
}

int main() {
  const unsigned ns[] = {1, 2, 3, 7, 31, 64, 100, 1000, 4096};
  const unsigned splits[] = {1, 2, 3, 8};
  const unsigned grids[] = {1, 5, 152, 608};
  long cases = 0;
  for (unsigned n : ns)
    for (unsigned split : splits)
      for (unsigned grid : grids) {
        const unsigned lags[] = {0u, 1u, n / 2, n > grid ? n - grid : 0u, grid, 2 * grid, n, n + 5};
        for (unsigned lag : lags) {
          const int r = check(n, split, lag, grid);
          if (r) {
            std::printf("fail %d: n=%u split=%u lag=%u grid=%u\n", r, n, split, lag, grid);
            return 1;
          }
          ++cases;
        }
      }
  std::printf("ok %ld\n", cases);
  return 0;
}
"""


def test_overlap_ticket_order(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "check.cpp"
    src.write_text(CHECK)
    exe = tmp_path / "check"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ")
