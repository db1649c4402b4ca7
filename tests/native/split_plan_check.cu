// Host-side walker over the split GEMM's planner (plan_build, compiled for the
// host from the same source as the kernels).  For every slice count 2..12,
// band width 1..4 and a spread of K it checks that the program issues each
// product A_i B_j with i + j <= s + 1 exactly once per K block, that every MMA's
// tile and TMEM indices are in range (wide MMAs start at an even buffer and
// cover two adjacent levels), that a stage never exceeds STAGE_TILES tiles,
// that each round respects the exact-FP32 budget s * kchunk * 256 <= 2^24,
// that continuation chains between groups are well formed, and that within a
// band every TMEM buffer is acquired once before its first MMA and released
// once after its last, and that the split-K chunk cap for products with few
// output tiles yields the chunk count the host expects, and that the row
// parts of a pipelined host-buffer product tile A in order, none empty.  Exit
// status 0 on success.  Launches no kernel.
#include "../../flag4j_gb300/csrc/f4j_split.cu"
#include <cstdio>
#include <set>
int main() {
  static SplitPlan P;
  int bad = 0;
  for (int band = 1; band <= 4; band++)
  for (int s = 2; s <= 12; s++) for (long long K : {64LL, 128LL, 1000LL, 8192LL, 16384LL, 70000LL, 200000LL, 1LL << 22}) {
    long long Kp = (K + BKB - 1) / BKB * BKB;
    int nr = plan_build(s, Kp, K, &P, band);
    if (nr < 0) { printf("overflow s=%d K=%lld band=%d\n", s, K, band); bad++; continue; }
    if (nr != s) { printf("rounds %d != levels %d\n", nr, s); bad++; }
    long long kchunk = (long long)P.kcb * BKB;
    if (P.kcb > 1 && (long long)s * kchunk * 256 > (1LL << 24)) { printf("exactness budget\n"); bad++; }
    if (P.kcb > P.nkb || P.nkb != Kp / BKB) { printf("chunking\n"); bad++; }
    std::multiset<int> seen;
    long long mmas = 0, instr = 0;
    int prev_out = 0, prev_r0 = -1;
    unsigned held = 0, acq_all = 0, rel_all = 0;
    for (int g = 0; g < P.ngroups; g++) {
      Group G = P.groups[g];
      const unsigned acq = ((unsigned)G.flags >> GF_ACQ_SHIFT) & 15u, rel = ((unsigned)G.flags >> GF_REL_SHIFT) & 15u;
      if (!(G.flags & GF_CONT_IN)) { held = 0; acq_all = 0; rel_all = 0; }
      if ((acq & acq_all) || (acq & held)) { printf("buffer acquired twice\n"); bad++; }
      held |= acq; acq_all |= acq;
      if (G.nr > NBUF || G.nr < 1) { printf("nr\n"); bad++; }
      if (G.nload > STAGE_TILES) { printf("stage size %d\n", G.nload); bad++; }
      bool cin = G.flags & GF_CONT_IN;
      if (cin != (prev_out != 0)) { printf("continuation chain\n"); bad++; }
      if (cin && G.r0 != prev_r0) { printf("continuation rounds\n"); bad++; }
      prev_out = G.flags & GF_CONT_OUT; prev_r0 = G.r0;
      for (int o = 0; o < G.nop; o++) {
        Op O = P.ops[G.op0 + o];
        const int U = TILE_BYTES >> 4;
        if (O.a_off % U || O.b_off % U || O.dcol % BN) { printf("op alignment\n"); bad++; continue; }
        const bool wide = O.idesc == umma_idesc_e4m3_f32(BM, 2 * BN);
        if (!wide && O.idesc != umma_idesc_e4m3_f32(BM, BN)) { printf("instruction descriptor\n"); bad++; }
        int la = O.a_off / U, lb = O.b_off / U, b0 = O.dcol / BN, nprod = wide ? 2 : 1;
        if (wide && (b0 % 2)) { printf("wide op at odd buffer\n"); bad++; }
        for (int u = 0; u < nprod; u++) {
          if (la >= G.nload || lb + u >= G.nload || b0 + u >= G.nr) { printf("op index\n"); bad++; continue; }
          Load a = P.loads[G.load0 + la], b = P.loads[G.load0 + lb + u];
          if (a.which != 0 || b.which != 1) { printf("operand kind\n"); bad++; }
          Round R = P.rounds[G.r0 + b0 + u];
          if (R.buf != b0 + u) { printf("round buffer\n"); bad++; }
          if (!((held >> (b0 + u)) & 1)) { printf("op on a buffer not held\n"); bad++; }
          int i = a.slice + 1, j = b.slice + 1;
          if (i + j != R.level || i < R.i0 || i >= R.i1) { printf("op level mismatch\n"); bad++; }
          seen.insert(i * 64 + j);
          mmas += 1;
        }
        instr++;
      }
      if ((rel & ~held) || (rel & rel_all)) { printf("release of a buffer not held\n"); bad++; }
      held &= ~rel; rel_all |= rel;
      if (!(G.flags & GF_CONT_OUT)) {
        const unsigned all = (1u << G.nr) - 1u;
        if (held || acq_all != all || rel_all != all) { printf("band buffers not acquired and released once\n"); bad++; }
      }
    }
    if (prev_out) { printf("dangling continuation\n"); bad++; }
    for (int r = 0; r < nr; r++)
      if (P.rounds[r].i1 - P.rounds[r].i0 > s) { printf("pairs per round\n"); bad++; }
    long long expect = 0;
    for (int i = 1; i <= s; i++) for (int j = 1; j <= s; j++) if (i + j <= s + 1) {
      expect++;
      if (seen.count(i * 64 + j) != 1) { printf("coverage (%d,%d) x%zu s=%d band=%d\n", i, j, seen.count(i*64+j), s, band); bad++; }
    }
    if ((long long)seen.size() != expect) { printf("coverage size\n"); bad++; }
  }
  // split K for few output tiles: the planner's chunk under the host's cap gives
  // exactly the chunk count the host sized the work units and workspace for,
  // for every slice count; many tiles or K > 64 blocks leave the plan alone
  for (long long tiles : {1LL, 8LL, 48LL, 64LL, 100LL, 151LL, 152LL, 4096LL})
  for (long long K : {64LL, 100LL, 128LL, 512LL, 1000LL, 1024LL, 1536LL, 2048LL, 4096LL, 4097LL, 8192LL}) {
    long long Kp = (K + BKB - 1) / BKB * BKB, nkb = Kp / BKB;
    int nch = 0;
    const int cap = split_kcb_cap(tiles, nkb, &nch);
    if ((tiles >= SPLIT_UNITS || nkb > 64) && (cap || nch)) { printf("split K outside its range\n"); bad++; }
    for (int s = 2; s <= 12; s++) {
      plan_build(s, Kp, K, &P, NBUF, cap);
      const long long pch = (P.nkb + P.kcb - 1) / P.kcb;
      if (cap && P.kcb != cap) { printf("chunk %d != cap %d (tiles %lld K %lld s %d)\n", P.kcb, cap, tiles, K, s); bad++; }
      if (nch && pch != nch) { printf("chunks %lld != %d\n", pch, nch); bad++; }
      if (cap && !nch && pch != 1) { printf("unsplit plan with %lld chunks\n", pch); bad++; }
    }
    if (tiles == 64 && K == 1024) printf("1024^3 (64 tiles, 16 K blocks): chunk %d blocks, %d chunks\n", cap, nch);
  }
  // ops per loaded tile for the default band
  for (int s : {8, 10, 11, 12}) {
    plan_build(s, 8192, 8192, &P, NBUF);
    int ops = 0, tiles = 0;
    for (int g = 0; g < P.ngroups; g++) { ops += P.groups[g].nop; tiles += P.groups[g].nload; }
    printf("s=%d: %d groups, %d MMA instructions for %d products, %d tiles per K block; kcb %d of %d\n", s, P.ngroups, ops, s*(s+1)/2, tiles, P.kcb, P.nkb);
  }
  // row parts of a pipelined host-buffer product: every tile-row count and
  // part count gives parts that tile [0, tiles_m) in order, none empty; the
  // first part has min(8, max(1, tiles_m / 4)) tile rows where that leaves a
  // row for each later part
  for (int tm = 1; tm <= 300; tm++)
    for (int parts = 1; parts <= F4J_HOST_PARTS_MAX && parts <= tm; parts++) {
      int b[F4J_HOST_PARTS_MAX + 1];
      host_part_bounds(tm, parts, b);
      if (b[0] != 0 || b[parts] != tm) { printf("parts %d of %d: ends %d, %d\n", parts, tm, b[0], b[parts]); bad++; }
      for (int p = 0; p < parts; p++)
        if (b[p + 1] <= b[p]) { printf("parts %d of %d: part %d empty\n", parts, tm, p); bad++; }
      const int a0 = tm / 4 < 1 ? 1 : (tm / 4 > 8 ? 8 : tm / 4);
      if (parts >= 2 && a0 <= tm - (parts - 1) && b[1] != a0) { printf("parts %d of %d: first %d\n", parts, tm, b[1]); bad++; }
    }
  printf("plan check: %s (%d problems)\n", bad ? "FAIL" : "ok", bad);
  return bad != 0;
}
