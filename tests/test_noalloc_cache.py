"""The per-context address cache behind ff_parsevalsum2_noalloc (csrc/ff_ctx_cache.h), on
the CPU: one lookup per context ID, a fresh lookup for a new ID (what a device reset or a
re-created primary context produces), and correct answers after the table is full."""
import os
import shutil
import subprocess

import pytest

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "fourierflows", "jl_gb300", "csrc")

PROG = r"""
#include <stdio.h>
#include <stdint.h>
#include "ff_ctx_cache.h"
int main() {
  ff::CtxAddressCache<4> c;
  int fetches = 0;
  auto fetch_for = [&](unsigned long long id) {
    return [&fetches, id](void** p) { ++fetches; *p = (void*)(uintptr_t)(0x1000 * id); return 0; };
  };
  void* p = nullptr;
  // the same context twice: one lookup
  if (c.get(7, &p, fetch_for(7)) || p != (void*)0x7000) return 1;
  if (c.get(7, &p, fetch_for(999)) || p != (void*)0x7000 || fetches != 1) return 2;
  // a re-created context (new ID) on the same device: a new lookup, not the stale address
  if (c.get(8, &p, fetch_for(8)) || p != (void*)0x8000 || fetches != 2) return 3;
  // a failing lookup is reported and not cached
  if (c.get(9, &p, [](void**) { return 700; }) != 700 || c.size() != 2) return 4;
  // more contexts than slots: every answer still belongs to its own context
  for (unsigned long long id = 10; id < 30; ++id)
    if (c.get(id, &p, fetch_for(id)) || p != (void*)(uintptr_t)(0x1000 * id)) return 5;
  if (c.size() != 4) return 6;
  const int before = fetches;
  if (c.get(29, &p, fetch_for(29)) || fetches != before) return 7;  // recent: cached
  if (c.get(7, &p, fetch_for(7)) || p != (void*)0x7000 || fetches != before + 1) return 8;  // evicted: fetched again
  printf("ok\n");
  return 0;
}
"""


def test_context_address_cache(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "cache_test.cpp"
    src.write_text(PROG)
    exe = tmp_path / "cache_test"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", HDR, str(src), "-o", str(exe), "-pthread"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
