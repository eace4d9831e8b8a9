"""The FP64 line kernels' job queues (csrc/plan.cpp build_schedule), on the host.

A small C++ program links the library, reads a case through the C ABI, builds the
plan and the queues for every launch-shape choice, and checks what the kernels rely
on: every chain of a launch's waves is in exactly one job; periodic chains run on a
whole warp; pairs hold two open chains, quads up to 8, bundles up to 32 open chains of
at most bundle_rows rows (longest first); no more warps than jobs; with the first wave's
first-sweep solve fused into the factorisation, exactly the factorisation queue's first-wave
jobs carry the fused flag."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "hamstr_oop_gb300", "csrc")
LIBDIR = os.path.join(ROOT, "hamstr_oop_gb300", "lib")

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "plan.h"
#include "hamstr_gpu.h"
using namespace hamstr;

static int fail(const char* what, int a, int b) { std::printf("FAIL %s %d %d\n", what, a, b); return 1; }

int main(int argc, char** argv) {
   hamstr_case* c = nullptr;
   char err[256];
   if (hamstr_case_open(argv[1], &c, err, sizeof err)) { std::printf("FAIL open %s\n", err); return 1; }
   if (argc > 2) hamstr_case_set_option(c, "chain_end_rule", 1);
   int sz[10];
   hamstr_case_sizes(c, sz);
   int nf = 0, ncc = 0, nfs = 0;
   hamstr_case_get_int(c, "faces", nullptr, &nf);
   hamstr_case_get_int(c, "chainConn", nullptr, &ncc);
   hamstr_case_get_int(c, "faceStartPerChain", nullptr, &nfs);
   std::vector<int> faces(nf), cc(ncc), fs(nfs);
   hamstr_case_get_int(c, "faces", faces.data(), nullptr);
   hamstr_case_get_int(c, "chainConn", cc.data(), nullptr);
   hamstr_case_get_int(c, "faceStartPerChain", fs.data(), nullptr);
   MeshInput in;
   in.nCell = sz[0]; in.nFace = sz[1]; in.nChain = sz[2]; in.nChainFace = fs[sz[2]];
   in.order = sz[5]; in.end_rule = argc > 2 ? END_RULE_EXTENDED : END_RULE_REFERENCE;
   in.faces = faces.data(); in.faceStartPerChain = fs.data(); in.chainConn = cc.data();
   Plan p;
   const std::string e = build_plan(in, p);
   if (!e.empty()) { std::printf("FAIL plan %s\n", e.c_str()); return 1; }
   int checked = 0, nper = 0, nspread = 0;
   for (int ch = 0; ch < p.nChain; ch++) nper += p.chain_periodic[ch];
   for (int maxw : {1, 7, 608})
    for (int spread : {0, 1})
      for (int lanes : {32, 16, 4})
         for (int br : {0, 2, 8, 64})
          for (int fuse : {0, 1}) {
            // nsm SMs with maxw / nsm warps each (0: long jobs not spread)
            const int nsm = spread ? (maxw == 608 ? 152 : maxw) : 0;
            const Schedule S = build_schedule(p, maxw, lanes, br, fuse != 0, 0, nsm);
            if ((int)S.njobs.size() != 1 + p.nWave) return fail("schedules", (int)S.njobs.size(), p.nWave);
            for (int s = 0; s <= p.nWave; s++) {
               std::vector<int> seen(p.nChain, 0);
               for (int k = 0; k < S.njobs[s]; k++) {
                  const int b = S.job_ptr[S.job0[s] + k], e2 = S.job_ptr[S.job0[s] + k + 1];
                  const int h = S.jobs[b] & ~kFusedJob;
                  // fused jobs: factorisation queue only, fusing on, chains of the first wave only
                  const bool fused = (S.jobs[b] & kFusedJob) != 0;
                  if (fused && (s != 0 || !fuse)) return fail("fused flag", s, fuse);
                  std::vector<int> ids;
                  if (h & kBundleJob) {
                     const int n = h & 63;
                     if (n < 1 || n > 32 || e2 - b != n + 1) return fail("bundle size", n, e2 - b);
                     for (int q = 1; q <= n; q++) ids.push_back(S.jobs[b + q]);
                     for (int id : ids)
                        if (p.chain_periodic[id] || p.chain_nrows[id] > br) return fail("bundle member", id, br);
                     if (p.chain_nrows[ids[0]] < p.chain_nrows[ids.back()]) return fail("bundle order", ids[0], 0);
                  } else if (h & kQuadJob) {
                     const int n = h & 63;
                     if (lanes != 4 || n < 1 || n > 8 || e2 - b != n + 1) return fail("quad size", n, e2 - b);
                     for (int q = 1; q <= n; q++) ids.push_back(S.jobs[b + q]);
                     for (int id : ids)
                        if (p.chain_periodic[id] || p.chain_nrows[id] <= br) return fail("quad member", id, br);
                  } else if (h & kPairJob) {
                     if (lanes != 16 || e2 - b != 2) return fail("pair size", e2 - b, lanes);
                     ids = {h & ~kPairJob, S.jobs[b + 1]};
                     for (int id : ids)
                        if (p.chain_periodic[id] || p.chain_nrows[id] <= br) return fail("pair member", id, br);
                  } else {
                     if (e2 - b != 1) return fail("single size", e2 - b, 0);
                     ids = {h};
                     if (!p.chain_periodic[h] && p.chain_nrows[h] <= br) return fail("single short open", h, br);
                  }
                  for (int id : ids) {
                     if (id < 0 || id >= p.nChain) return fail("chain id", id, p.nChain);
                     if (fused && p.chain_wave[id] != 0) return fail("fused wave", id, p.chain_wave[id]);
                     if (s == 0 && fuse && p.chain_wave[id] == 0 && !fused) return fail("first wave unfused", id, 0);
                     if (s > 0 && p.chain_wave[id] != s - 1) return fail("wave", id, s - 1);
                     seen[id]++;
                  }
               }
               for (int ch = 0; ch < p.nChain; ch++) {
                  const int want = (s == 0 || p.chain_wave[ch] == s - 1) ? 1 : 0;
                  if (seen[ch] != want) return fail("coverage", ch, seen[ch]);
               }
               const int nw = S.nwarps[s], base = S.njobs[s] < maxw ? S.njobs[s] : maxw;
               if ((int)S.ncrit.size() != 1 + p.nWave) return fail("outlier lists", (int)S.ncrit.size(), p.nWave);
               const int nc = S.ncrit[s];
               if (nc >= 0) {
                  // outliers alone on their SM, or nothing placed
                  if (nc > kMaxCrit || nc > S.njobs[s]) return fail("outlier jobs", nc, S.njobs[s]);
                  if (nw != base) return fail("warps", nw, S.njobs[s]);
               } else {
                  // long jobs spread one per SM, a block on each of those SMs
                  const int wpb = maxw / nsm;
                  if (nsm == 0 || -nc > S.njobs[s] || -nc > nsm || (-nc <= kMaxCrit && -nc != nsm))
                     return fail("spread jobs", nc, S.njobs[s]);
                  if (nw != std::max(base, std::min(-nc * wpb, maxw))) return fail("spread warps", nw, -nc);
                  if (nw > maxw || (nw + wpb - 1) / wpb < -nc) return fail("spread blocks", nw, -nc);
                  nspread++;
               }
               checked++;
            }
         }
   std::printf("OK %d %d %d %d %d\n", checked, p.nChain, nper, p.nWave, nspread);
   hamstr_case_close(c);
   return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory, native_lib):
    d = tmp_path_factory.mktemp("sched")
    src = d / "sched.cpp"
    src.write_text(PROGRAM)
    exe = d / "sched"
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", CSRC, "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", LIBDIR, "-lhamstr_gb300", "-Wl,-rpath," + LIBDIR, "-o", str(exe)], check=True)
    return str(exe)


@pytest.mark.parametrize("ni,nj,split,extended", [(32, 8, 0.0, False), (32, 12, 0.0, False), (128, 32, 0.0, False),
                                                   (24, 8, 0.5, True), (40, 10, 0.3, True)])
def test_line_job_queues(harness, make_case, ni, nj, split, extended):
    case = make_case(ni, nj, split=split, seed=4, order=3)
    args = [harness, case] + (["extended"] if extended else [])
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("OK"), out.stdout + out.stderr
    checked, nchain, nper, nwave, nspread = (int(x) for x in out.stdout.split()[1:])
    assert checked == 3 * 2 * 3 * 4 * 2 * (1 + nwave) and nchain > 0
    if split == 0.0:
        assert nper > 0                  # the plain O-grid has periodic loops beside open lines
    if nj > 8 and split == 0.0:
        assert nspread > 0               # more equal loops than outliers: spread one per SM


@pytest.mark.gpu
def test_row_wait_gives_up_at_its_bound(native_lib):
    """The shared-memory row count a line solve waits on behind its
    factorisation (line_solve.cuh publish_rows / wait_rows): waits for
    published rows are met, a wait for a row that is never published gives
    up at its bound instead of spinning on, and the kernel ends."""
    import ctypes
    import time
    import torch
    out = torch.full((3,), -1, dtype=torch.int32, device="cuda")
    fn = native_lib.hamstr_check_row_wait
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    t0 = time.perf_counter()
    assert fn(out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 30
    assert out.cpu().tolist() == [1, 1, 0]
