"""The host-thread split the runtime uses for the negative sampler
(`parallel_indices` in distembed_gb300/csrc/de_internal.h), compiled on the CPU:
every index of [0, count) is visited exactly once, below and above the size at
which it starts threads, and the draws it produces match a serial loop."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = next((d for d in (os.environ.get("CUDA_HOME", "") + "/include", "/usr/local/cuda/include")
                 if os.path.exists(os.path.join(d, "cuda_runtime.h"))), None)

PROGRAM = r"""
#include <atomic>
#include <cstdio>
#include <random>
#include <vector>
#include "de_internal.h"

int main() {
  // coverage: each index once, for counts around the threading threshold
  for (long long count : {0LL, 1LL, 7LL, 1000LL, 262143LL, 262144LL, 1000003LL}) {
    std::vector<std::atomic<int>> hits(count);
    for (auto &h : hits) h = 0;
    de::parallel_indices(count, 1, [&](int64_t i) { hits[i].fetch_add(1); });
    for (long long i = 0; i < count; ++i)
      if (hits[i] != 1) { std::printf("count %lld index %lld hit %d times\n", count, i, int(hits[i])); return 1; }
  }
  // the sampler's draws (seed = epoch + minibatch), threaded against serial
  const int epochs = 10, batches = 512, ns = 1024;
  const long long n = 4194304;
  std::vector<int> serial(size_t(epochs) * batches * ns), threaded(serial.size());
  auto draw = [&](int64_t q, int *out) {
    std::minstd_rand gen(int(q / batches) + int(q % batches));
    std::uniform_int_distribution<int> dist(0, int(n));
    for (int k = 0; k < ns; ++k) out[k] = dist(gen);
  };
  for (int64_t q = 0; q < int64_t(epochs) * batches; ++q) draw(q, serial.data() + q * ns);
  de::parallel_indices(int64_t(epochs) * batches, ns, [&](int64_t q) { draw(q, threaded.data() + q * ns); });
  if (serial != threaded) { std::printf("threaded draws differ\n"); return 1; }
  std::printf("ok\n");
  return 0;
}
"""


@pytest.mark.skipif(CUDA_INC is None or shutil.which("g++") is None, reason="needs g++ and the CUDA headers")
def test_parallel_indices_visits_each_index_once(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "t"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "distembed_gb300", "csrc"),
                           "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC, str(src), "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
