// ##################################################################
//
// plan.cpp -- derive the per-mesh kernel layout from the chain files
//
// Follows the reference's per-call logic once, up front:
//   stencil + ghosts   computeRHS.cpp:57-149, :154-260
//   face order         computeRHS.cpp:278-408
//   block assembly     ADI.cpp:62-217
//   chain order        ADI.cpp:57 (file order; realised as waves of
//                      cell-disjoint chains that commute)
// ##################################################################
#include "plan.h"

#include <algorithm>
#include <cstdio>
#include <unordered_map>

namespace hamstr {

namespace {

std::string fmt(const char* f, int a, int b = 0)
{
   char buf[256];
   std::snprintf(buf, sizeof(buf), f, a, b);
   return buf;
}

struct BlockOps {
   int op[kOpsPerBlock];
   int n = 0;
   BlockOps() { for (int& o : op) o = -1; }
   bool add(int v)
   {
      if (n >= kOpsPerBlock) return false;
      op[n++] = v;
      return true;
   }
};

}  // namespace

std::string build_plan(const MeshInput& in, Plan& p)
{
   p = Plan();
   p.nCell = in.nCell;
   p.nFace = in.nFace;
   p.nChain = in.nChain;
   p.order = in.order;
   if (in.order != 1 && in.order != 3 && in.order != 5)
      return fmt("unsupported reconstruction order %d", in.order);
   p.nGhost = (in.order == 5) ? 3 : 2;
   const int g = p.nGhost;
   if (in.nCell <= 0 || in.nFace <= 0 || in.nChain <= 0) return "empty mesh";
   auto left_of = [&](int face) { return in.faces[6 * face + 2]; };
   auto right_of = [&](int face) { return in.faces[6 * face + 4]; };

   // ---- validation of ids ------------------------------------------
   for (int i = 0; i < in.nFace; i++) {
      int l = left_of(i), r = right_of(i);
      if (l < 0 || l >= in.nCell) return fmt("face %d has invalid left cell %d", i, l);
      if (r >= in.nCell) return fmt("face %d has invalid right cell %d", i, r);
      if (r == -5) return fmt("face %d is an inter-domain face (not supported)", i);
      if (r < -2) return fmt("face %d has unknown boundary tag %d", i, r);
   }
   for (int c = 0; c <= in.nChain; c++) {
      int s = in.faceStartPerChain[c];
      if (s < 0 || s > in.nChainFace) return fmt("chain offset %d out of range (%d)", c, s);
      if (c > 0 && s <= in.faceStartPerChain[c - 1]) return fmt("chain %d is empty or reversed", c - 1);
   }
   for (int f = 0; f < in.nChainFace; f++)
      if (in.chainConn[f] < 0 || in.chainConn[f] >= in.nFace)
         return fmt("chain face entry %d is not a face (%d)", f, in.chainConn[f]);

   // ---- stencils and slots -----------------------------------------
   // Under END_RULE_EXTENDED an open chain's ghosts are set by position:
   // the k-th ghost beyond an end face holds the neighbour across an
   // interior face, the wall mirror of the k-th cell from that end (the
   // last one on shorter chains), or the freestream.  The reference's rule
   // reads ghost ids that the chain itself never wrote when an open chain
   // has fewer than nGhost (order 5) or 2 cells, so such chains are
   // rejected there.
   const bool ext = in.end_rule == END_RULE_EXTENDED;
   if (in.end_rule != END_RULE_REFERENCE && !ext) return fmt("unknown chain end rule %d", in.end_rule);
   std::vector<int>& chain_sten0 = p.chain_sten0;
   chain_sten0.assign(in.nChain, 0);
   std::vector<int> ci;
   std::vector<int> face_last_slot(in.nFace, -1);
   for (int ich = 0; ich < in.nChain; ich++) {
      const int f1 = in.faceStartPerChain[ich], f2 = in.faceStartPerChain[ich + 1];
      const int nf = f2 - f1;
      const bool closed = in.chainConn[f1] == in.chainConn[f2 - 1];
      if (closed && (nf < 3 || nf < g + 1)) return fmt("closed chain %d too short (%d faces)", ich, nf);
      if (!closed && nf < 2) return fmt("open chain %d too short (%d faces)", ich, nf);
      if (!closed && !ext && nf - 1 < (g == 3 ? 3 : 2))
         return fmt("open chain %d has %d cells: the reference's ghost rule needs more "
                    "(use the extended chain end rule)", ich, nf - 1);
      ci.assign(nf + 2 * g + 2, 0);
      int m = g, size;
      for (int f = f1; f < f2; f++) ci[m++] = left_of(in.chainConn[f]);
      if (closed) {
         ci[m++] = left_of(in.chainConn[f1 + 1]);
         size = m;
         m = 0;
         for (int f = f2 - g - 1; f < f2 - 1; f++) ci[m++] = left_of(in.chainConn[f]);
      } else if (g == 3) {
         m--; ci[m] = -ci[m];
         m++; ci[m] = -ci[m - 3];
         m++; ci[m] = -ci[m - 5];
         size = m + 1;
         ci[0] = -ci[5];
         ci[1] = -ci[4];
         ci[2] = -ci[3];
      } else {
         m--; ci[m] = -ci[m];
         m++; ci[m] = -ci[m - 3];
         size = m + 1;
         ci[0] = -ci[3];
         ci[1] = -ci[2];
      }
      chain_sten0[ich] = (int)p.sten_cell.size();
      if (ext && !closed) {
         const int n = size - 2 * g;
         auto ghost = [&](int iface, int mc) {
            const int right = right_of(iface);
            if (right >= 0) {
               p.sten_cell.push_back(right);
               p.sten_kind.push_back(STEN_CELL);
               p.sten_face.push_back(-1);
            } else if (right == -2) {
               p.sten_cell.push_back(mc);
               p.sten_kind.push_back(STEN_WALL);
               p.sten_face.push_back(iface);
            } else {
               p.sten_cell.push_back(-1);
               p.sten_kind.push_back(STEN_FREESTREAM);
               p.sten_face.push_back(-1);
            }
         };
         for (int k = g; k >= 1; k--) ghost(in.chainConn[f1], ci[g + std::min(k - 1, n - 1)]);
         for (int j = g; j < g + n; j++) {
            p.sten_cell.push_back(ci[j]);
            p.sten_kind.push_back(STEN_CELL);
            p.sten_face.push_back(-1);
         }
         for (int k = 1; k <= g; k++) ghost(in.chainConn[f2 - 1], ci[g + n - 1 - std::min(k - 1, n - 1)]);
      }
      for (int j = 0; j < size && !(ext && !closed); j++) {
         const int icell = ci[j];
         const bool ghost = icell < 0 || (icell == 0 && (j == g - 1 || j == size - g));
         int kind = STEN_CELL, cell = icell, face = -1;
         if (ghost) {
            const int iface = (j < g) ? in.chainConn[f1] : in.chainConn[f2 - 1];
            const int right = right_of(iface);
            if (right == -2) {
               kind = STEN_WALL;
               cell = -icell;
               face = iface;
            } else {
               kind = STEN_FREESTREAM;
               cell = -1;
            }
         }
         if (kind != STEN_FREESTREAM && (cell < 0 || cell >= in.nCell))
            return fmt("chain %d stencil slot %d names no cell", ich, j);
         p.sten_cell.push_back(cell);
         p.sten_kind.push_back(kind);
         p.sten_face.push_back(face);
      }
      // processed faces (computeRHS.cpp:278-281)
      const int per = closed ? 1 : 0;
      for (int f = f1; f < f2 - per; f++) {
         const int iface = in.chainConn[f];
         const int s = (int)p.slot_face.size();
         p.slot_face.push_back(iface);
         p.slot_left.push_back(left_of(iface));
         p.slot_right.push_back(right_of(iface));
         p.slot_n.push_back(chain_sten0[ich] + (g - 1) + (f - f1));
         p.slot_swap.push_back((f == f2 - 1 && !closed) ? 1 : 0);
         face_last_slot[iface] = s;
      }
   }
   p.nSten = (int)p.sten_cell.size();
   p.nSlot = (int)p.slot_face.size();
   p.slot_owner.resize(p.nSlot);
   for (int s = 0; s < p.nSlot; s++) p.slot_owner[s] = face_last_slot[p.slot_face[s]];

   // ---- per-cell ordered contributions -----------------------------
   std::vector<int> cnt(in.nCell + 1, 0);
   for (int s = 0; s < p.nSlot; s++) {
      cnt[p.slot_left[s] + 1]++;
      if (p.slot_right[s] > -1) cnt[p.slot_right[s] + 1]++;
   }
   p.cell_ptr.assign(in.nCell + 1, 0);
   for (int c = 0; c < in.nCell; c++) p.cell_ptr[c + 1] = p.cell_ptr[c] + cnt[c + 1];
   p.cell_ent.assign(p.cell_ptr[in.nCell], 0);
   std::vector<int> fill(p.cell_ptr.begin(), p.cell_ptr.end() - 1);
   for (int s = 0; s < p.nSlot; s++) {
      p.cell_ent[fill[p.slot_left[s]]++] = 2 * s;
      if (p.slot_right[s] > -1) p.cell_ent[fill[p.slot_right[s]]++] = 2 * s + 1;
   }

   // ---- ADI rows (ADI.cpp:62-217) -----------------------------------
   // extended rule: chain-end faces whose right cell lies on another chain
   // (CSR over that cell, ascending face ids) and each cell's first chain
   std::vector<int> xptr(in.nCell + 1, 0), xent, first_chain(in.nCell, -1);
   if (ext) {
      std::vector<char> isend(in.nFace, 0);
      for (int ich = 0; ich < in.nChain; ich++) {
         const int a = in.chainConn[in.faceStartPerChain[ich]];
         const int b = in.chainConn[in.faceStartPerChain[ich + 1] - 1];
         if (a == b) continue;
         isend[a] = isend[b] = 1;
      }
      for (int f = 0; f < in.nFace; f++)
         if (isend[f] && right_of(f) >= 0) xptr[right_of(f) + 1]++;
      for (int c = 0; c < in.nCell; c++) xptr[c + 1] += xptr[c];
      xent.assign(xptr[in.nCell], 0);
      std::vector<int> xf(xptr.begin(), xptr.end() - 1);
      for (int f = 0; f < in.nFace; f++)
         if (isend[f] && right_of(f) >= 0) xent[xf[right_of(f)]++] = f;
      for (int ich = in.nChain - 1; ich >= 0; ich--)
         for (int f = in.faceStartPerChain[ich]; f < in.faceStartPerChain[ich + 1] - 1; f++)
            first_chain[left_of(in.chainConn[f])] = ich;
   }
   int slot0 = 0;
   std::vector<int> lastwave(in.nCell, -1);
   p.cell_last_wave_writer.assign(in.nCell, 0);
   for (int ich = 0; ich < in.nChain; ich++) {
      const int f1 = in.faceStartPerChain[ich], f2 = in.faceStartPerChain[ich + 1];
      const int per = (in.chainConn[f1] == in.chainConn[f2 - 1]) ? 1 : 0;
      const int nproc = f2 - per - f1;
      const int N = per ? nproc : nproc - 1;
      std::vector<BlockOps> A(nproc + 1), B(nproc + 1), C(nproc + 1);
      std::vector<int> fcell(nproc + 1, -1);
      int m = 0;
      bool ok = true;
      for (int f = f1; f < f2 - per; f++) {
         const int s = slot0 + (f - f1);
         const int own = p.slot_owner[s];
         const int iface = in.chainConn[f];
         const int right = right_of(iface);
         const int L = (own << 3) | (OP_SEL_L << 1), R = (own << 3) | (OP_SEL_R << 1);
         const int Rr = (own << 3) | (OP_SEL_RREFL << 1);
         if (per) {
            const int mm1 = (m == 0) ? nproc - 1 : m - 1;
            ok &= B[m].add(L);
            ok &= B[mm1].add(R | 1);
            ok &= A[m].add(R);
            ok &= C[mm1].add(L | 1);
            fcell[m] = left_of(iface);
         } else {
            const int mm1 = m - 1;
            // extended rule: an interior last face couples explicitly, like
            // the far field (the reference indexes a row past the chain)
            const bool ext_last = ext && f == f2 - 1;
            if ((right < 0 || ext_last) && f == f2 - 1) m--;
            ok &= B[m].add(L);
            if (mm1 > -1 && right > -1 && !ext_last) {
               ok &= A[m].add(R);
               ok &= B[mm1].add(R | 1);
               ok &= C[mm1].add(L | 1);
            } else if (right == -2) {
               ok &= B[m].add(Rr);
            }
            fcell[m] = left_of(iface);
         }
         m++;
      }
      if (ext) {
         // a cell's first chain also carries the diagonal term of each
         // chain-end face leading into it from another chain
         for (int r = 0; r < N; r++) {
            const int sc = left_of(in.chainConn[f1 + r]);
            if (first_chain[sc] != ich) continue;
            for (int e = xptr[sc]; e < xptr[sc + 1]; e++)
               ok &= B[r].add((p.slot_owner[face_last_slot[xent[e]]] << 3) | (OP_SEL_R << 1) | 1);
         }
      }
      if (!ok) return fmt("chain %d needs more than %d terms in one block", ich, kOpsPerBlock);
      p.chain_periodic.push_back(per);
      p.chain_nrows.push_back(N);
      p.chain_row0.push_back((int)p.row_scell.size());
      p.maxRows = std::max(p.maxRows, N);
      int wave = 0;
      for (int r = 0; r < N; r++) {
         const int sc = left_of(in.chainConn[f1 + r]);
         p.row_scell.push_back(sc);
         p.row_fcell.push_back(fcell[r]);
         for (int o = 0; o < kOpsPerBlock; o++) p.row_ops.push_back(A[r].op[o]);
         for (int o = 0; o < kOpsPerBlock; o++) p.row_ops.push_back(B[r].op[o]);
         for (int o = 0; o < kOpsPerBlock; o++) p.row_ops.push_back(C[r].op[o]);
         wave = std::max(wave, lastwave[sc] + 1);
         if (fcell[r] >= 0) wave = std::max(wave, lastwave[fcell[r]] + 1);
      }
      for (int r = 0; r < N; r++) {
         const int sc = p.row_scell[p.chain_row0.back() + r];
         lastwave[sc] = std::max(lastwave[sc], wave);
         p.cell_last_wave_writer[sc] = 1;
         const int fc = p.row_fcell[p.chain_row0.back() + r];
         if (fc >= 0) lastwave[fc] = std::max(lastwave[fc], wave);
      }
      p.chain_wave.push_back(wave);
      p.nWave = std::max(p.nWave, wave + 1);
      slot0 += nproc;
   }
   p.nRow = (int)p.row_scell.size();
   p.wave_ptr.assign(p.nWave + 1, 0);
   for (int w : p.chain_wave) p.wave_ptr[w + 1]++;
   for (int w = 0; w < p.nWave; w++) p.wave_ptr[w + 1] += p.wave_ptr[w];
   p.wave_chains.assign(in.nChain, 0);
   std::vector<int> wfill(p.wave_ptr.begin(), p.wave_ptr.end() - 1);
   for (int ich = 0; ich < in.nChain; ich++) p.wave_chains[wfill[p.chain_wave[ich]]++] = ich;
   return "";
}

Schedule build_schedule(const Plan& p, int max_warps, int open_lanes, int bundle_rows, bool fuse_first_wave,
                        int max_warps_factor, int nsm)
{
   Schedule S;
   S.job_ptr.push_back(0);
   // jobs ordered by their estimated time, longest first: a row of a warp,
   // half-warp or four-lane form is a chain of dependent FP64 operations
   // (latency; the factorisation's block LU about three times the solve's),
   // a row of a bundle is ~274 (factorisation) or ~92 (solve) FP64 warp
   // instructions issued back to back
   struct Job { double cost; std::vector<int> entries; };
   // the jobs of one chain set, with their cost per row of the longest chain
   auto pack = [&](const std::vector<int>& chains, double row_warp, double row_bundle) {
      std::vector<int> sorted(chains);
      std::stable_sort(sorted.begin(), sorted.end(),
                       [&](int a, int b) { return p.chain_nrows[a] > p.chain_nrows[b]; });
      std::vector<Job> order;
      std::vector<int> bundle, group;
      auto flush = [&](std::vector<int>& v, int flag, double row_cost) {
         if (v.empty()) return;
         Job j;
         j.cost = row_cost * p.chain_nrows[v.front()];   // longest first
         if (flag == kPairJob && v.size() == 2) {
            j.entries = {v[0] | kPairJob, v[1]};
         } else if (flag == kPairJob || flag == 0) {
            j.entries = {v[0]};
         } else {
            j.entries.push_back(flag | (int)v.size());
            j.entries.insert(j.entries.end(), v.begin(), v.end());
         }
         order.push_back(j);
         v.clear();
      };
      const int group_size = open_lanes == 4 ? 8 : open_lanes == 16 ? 2 : 1;
      const int group_flag = open_lanes == 4 ? kQuadJob : open_lanes == 16 ? kPairJob : 0;
      for (int c : sorted) {
         const int n = p.chain_nrows[c];
         if (p.chain_periodic[c]) {
            order.push_back({1.3 * row_warp * n, {c}});
         } else if (n <= bundle_rows) {
            bundle.push_back(c);
            if ((int)bundle.size() == 32) flush(bundle, kBundleJob, row_bundle);
         } else {
            group.push_back(c);
            if ((int)group.size() == group_size) flush(group, group_flag, row_warp);
         }
      }
      flush(bundle, kBundleJob, row_bundle);
      flush(group, group_flag, row_warp);
      return order;
   };
   auto emit = [&](std::vector<Job>& order, int maxw) {
      std::stable_sort(order.begin(), order.end(), [](const Job& x, const Job& y) { return x.cost > y.cost; });
      S.job0.push_back((int)S.job_ptr.size() - 1);
      S.njobs.push_back((int)order.size());
      int nw = std::min((int)order.size(), maxw);
      int nc = 0;
      while (nc < (int)order.size() && order[nc].cost >= kCritFrac * order[0].cost) nc++;
      if (nc <= kMaxCrit) {
         S.ncrit.push_back(nc);
      } else if (nsm > 0) {
         // many long jobs: one per SM, and a block on every SM that holds one
         const int spread = std::min(nc, nsm), wpb = std::max(1, maxw / nsm);
         S.ncrit.push_back(-spread);
         nw = std::max(nw, std::min(spread * wpb, maxw));
      } else {
         S.ncrit.push_back(0);
      }
      S.nwarps.push_back(nw);
      for (const Job& j : order) {
         S.jobs.insert(S.jobs.end(), j.entries.begin(), j.entries.end());
         S.job_ptr.push_back((int)S.jobs.size());
      }
   };
   auto wave = [&](int w) {
      return std::vector<int>(p.wave_chains.begin() + p.wave_ptr[w], p.wave_chains.begin() + p.wave_ptr[w + 1]);
   };
   constexpr double kFacWarp = 6.0, kFacBundle = 22.0, kSolWarp = 2.0, kSolBundle = 7.4;
   // schedule 0, the factorisation: all chains; fused, the first wave's jobs
   // are packed as its solve packs them and carry that solve as well
   std::vector<Job> fac;
   if (fuse_first_wave && p.nWave > 0) {
      fac = pack(wave(0), kFacWarp + kSolWarp, kFacBundle + kSolBundle);
      for (Job& j : fac) j.entries[0] |= kFusedJob;
      std::vector<int> rest(p.wave_chains.begin() + p.wave_ptr[1], p.wave_chains.end());
      std::vector<Job> more = pack(rest, kFacWarp, kFacBundle);
      fac.insert(fac.end(), more.begin(), more.end());
   } else {
      std::vector<int> all(p.nChain);
      for (int c = 0; c < p.nChain; c++) all[c] = c;
      fac = pack(all, kFacWarp, kFacBundle);
   }
   emit(fac, max_warps_factor > 0 ? max_warps_factor : max_warps);
   for (int w = 0; w < p.nWave; w++) {
      std::vector<Job> sol = pack(wave(w), kSolWarp, kSolBundle);
      emit(sol, max_warps);
   }
   return S;
}

}  // namespace hamstr
