"""Once-per-device setup shared by host threads (openblas_gb300/csrc/per_device.h).

The library sets kernel attributes and caches occupancy figures and the SM
count once per device.  The helper that does this is plain C++, so it is
compiled here with g++ into a small program that runs it from many threads
at once.  The program checks that:
- each device's step ran exactly once;
- no caller went on before that step had finished;
- a failed step is retried and its status reaches the caller;
- cached values are per device;
- an ordinal outside the table runs the step every time.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>
#include "per_device.h"

static std::atomic<int> ran[8];
static std::atomic<int> finished[8];
static std::atomic<int> early{0};

int main() {
  gb::PerDeviceOnce once;
  gb::PerDeviceValue<int> value;
  std::vector<std::thread> threads;
  for (int t = 0; t < 32; ++t)
    threads.emplace_back([&, t] {
      for (int rep = 0; rep < 200; ++rep) {
        const int dev = (int)((unsigned)(t + rep) % 8u);
        const int st = once.run(dev, [&] {
          ran[dev]++;
          std::this_thread::sleep_for(std::chrono::milliseconds(2));
          finished[dev] = 1;
          return 0;
        });
        if (st != 0 || !finished[dev]) early++;
        if (value.get(dev, [dev] { return 100 + dev; }) != 100 + dev) early++;
      }
    });
  for (auto &th : threads) th.join();
  for (int d = 0; d < 8; ++d)
    if (ran[d] != 1) { printf("device %d ran %d times\n", d, (int)ran[d]); return 1; }
  if (early) { printf("%d callers went on early or saw a wrong value\n", (int)early); return 2; }

  gb::PerDeviceOnce flaky;
  int tries = 0;
  auto step = [&] { return ++tries < 3 ? 7 : 0; };
  if (flaky.run(0, step) != 7 || flaky.run(0, step) != 7 || flaky.run(0, step) != 0 ||
      flaky.run(0, step) != 0 || tries != 3) { printf("retry: tries %d\n", tries); return 3; }

  int outside = 0;
  for (int i = 0; i < 5; ++i) once.run(64, [&] { ++outside; return 0; });
  if (outside != 5) { printf("ordinal 64 ran %d times\n", outside); return 4; }
  printf("ok\n");
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_per_device_once_under_threads(tmp_path):
    src = tmp_path / "per_device_check.cpp"
    exe = tmp_path / "per_device_check"
    src.write_text(PROGRAM)
    inc = os.path.join(ROOT, "openblas_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I", inc, str(src), "-o", str(exe)],
                   check=True, capture_output=True, timeout=120)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok"
