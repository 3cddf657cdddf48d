// Host-side check of the tensor-core block kernel's index tables.
//
// Includes qgb_tc.cu and replays k_fused5_tc's data movement on the CPU with
// the tables make_geom builds: the coalesced load (thread t, step r -> global
// offset), the A operand layout (decoded back to (group row, column)), the
// permuted block product in FP64, the staging slots of the epilogue and the
// coalesced store.  For n = 5..16 and random, lowest and highest block-qubit
// placements it checks that every amplitude is read and written exactly
// once, that every shared-memory offset lies inside its buffer and is used
// once, and that the result equals the block applied directly.  It also
// counts shared-memory wavefronts per warp access (8-byte accesses, one
// wavefront per half-warp without conflicts) and fails if any pattern needs
// more than the layout promises: 2 per warp for the staging writes and
// reads, 2 for A writes of blocks with a qubit on index bits 0..3, else 4.
// The tensor-memory variant k_fused5_tcm is replayed the same way with the
// tables of make_geom_m.  No kernel is launched.
#include <complex>
#include <cstring>
#include <cstdio>
#include <map>
#include <random>
#include <set>

#include "qgb_tc.cu"

typedef std::complex<double> cd;

static i64 host_tile_base(i64 t, const TcGeom& geo) {
  i64 base = 0;
  for (int b = 0; b < geo.nrest; ++b) base |= ((t >> b) & 1) << geo.rest[b];
  return base;
}

// wavefronts of one warp of 8-byte shared-memory accesses (byte offsets)
static int wavefronts(const uint32_t* off) {
  int total = 0;
  for (int h = 0; h < 2; ++h) {
    std::map<int, std::set<uint32_t>> bank;
    for (int l = 16 * h; l < 16 * h + 16; ++l) {
      bank[(off[l] / 4) % 32].insert(off[l] / 4);
      bank[(off[l] / 4 + 1) % 32].insert(off[l] / 4 + 1);
    }
    int m = 0;
    for (auto& kv : bank) m = std::max<int>(m, (int)kv.second.size());
    total += m;
  }
  return total;
}

static cd block_row(const std::vector<zd>& U, const int idx[32], int r, const cd* x) {
  cd acc = 0;
  for (int k = 0; k < 32; ++k) {
    const zd u = U[idx[r] * 32 + idx[k]];
    acc += cd(u.real(), u.imag()) * x[k];
  }
  return acc;
}

// k_fused5_tcm on the CPU with the tables make_geom_m builds: thread (warp
// w, lane l) loads its row's 16 amplitudes of column half w / 4, the
// permuted block product runs per row, and each thread stores its outputs
// to the addresses it loaded.  Every amplitude must be read and written
// once and the result must equal the block applied directly.
// tcm_transpose on the host: exchange lane bit i with register bit i for
// i < nswap, a shuffle being a read of the partner lane's value
template <typename V>
static void host_tcm_transpose(V (&v)[32][16], int nswap) {
  for (int i = 0; i < nswap; ++i) {
    V nv[32][16];
    for (int l = 0; l < 32; ++l)
      for (int r = 0; r < 16; ++r) nv[l][r] = v[l][r];
    for (int l = 0; l < 32; ++l) {
      const bool up = (l >> i) & 1;
      const int p = l ^ (1 << i);
      for (int r = 0; r < 16; ++r) {
        if (r & (1 << i)) continue;
        const int r1 = r | (1 << i);
        const bool pup = !up;
        const V recv = pup ? v[p][r] : v[p][r1];  // what lane p sends
        if (up) nv[l][r] = recv;
        else nv[l][r1] = recv;
      }
    }
    for (int l = 0; l < 32; ++l)
      for (int r = 0; r < 16; ++r) v[l][r] = nv[l][r];
  }
}

static int check_tcm(std::mt19937_64& rng) {
  std::normal_distribution<double> nd;
  int fails = 0;
  for (int n = 12; n <= 16; ++n) {
    for (int trial = 0; trial < 16; ++trial) {
      std::vector<int> all(n);
      for (int i = 0; i < n; ++i) all[i] = i;
      std::shuffle(all.begin(), all.end(), rng);
      std::vector<int> tb(all.begin(), all.begin() + 5);
      if (trial == 0) tb = {n - 1, n - 2, n - 3, n - 4, n - 5};
      if (trial == 1) tb = {4, 3, 2, 1, 0};
      if (trial == 2) tb = {9, 0, 2, 6, 5};
      if (trial == 3) tb = {1, 0, 8, 3, 2};
      if (trial == 4) tb = {11, 1, 4, 3, 2};
      if (trial == 5) tb = {0, 1, 7, 10, 11};
      std::vector<zd> U(1024);
      for (auto& c : U) c = zd(nd(rng), nd(rng));
      const i64 N = (i64)1 << n;
      std::vector<cd> psi(N), ref(N);
      for (auto& x : psi) x = cd(nd(rng), nd(rng));
      for (i64 i = 0; i < N; ++i) {
        int bi = 0;
        for (int jt = 0; jt < 5; ++jt) bi |= (int)((i >> tb[jt]) & 1) << (4 - jt);
        if (bi) continue;
        i64 id[32];
        for (int b = 0; b < 32; ++b) {
          id[b] = i;
          for (int jt = 0; jt < 5; ++jt)
            if ((b >> (4 - jt)) & 1) id[b] |= (i64)1 << tb[jt];
        }
        for (int r = 0; r < 32; ++r) {
          cd acc = 0;
          for (int c = 0; c < 32; ++c) acc += cd(U[r * 32 + c].real(), U[r * 32 + c].imag()) * psi[id[c]];
          ref[id[r]] = acc;
        }
      }
      for (int shfl = 0; shfl < 2; ++shfl) {
        TcmGeom* gm = new TcmGeom();
        int cbit[5], idx[32];
        make_geom_m(n, tb, shfl != 0, gm, cbit);
        block_perm(cbit, idx);
        std::vector<cd> out(N, cd(1e300, 0));
        std::vector<int> seen(N, 0), wrote(N, 0);
        bool bad = gm->nrest != n - 12 || gm->nswap < 0 || gm->nswap > 4;
        int worst_lines = 0;
        for (i64 t = 0; t < ((i64)1 << (n - 12)) && !bad; ++t) {
          i64 base = 0;
          for (int b = 0; b < gm->nrest; ++b) base |= ((t >> b) & 1) << gm->rest[b];
          for (int w = 0; w < 8; ++w) {
            // the warp's loads, then the lane / register exchanges
            cd v[32][16];
            i64 addr[32][16];
            for (int l = 0; l < 32; ++l)
              for (int r = 0; r < 16; ++r) {
                const i64 gi = base + gm->lanes[l] + gm->rowhi[w & 3] + ((w >> 2) ? gm->chi : 0) + gm->clo[r];
                addr[l][r] = gi;
                if (gi < 0 || gi >= N) { bad = true; v[l][r] = 0; continue; }
                seen[gi]++;
                v[l][r] = psi[gi];
              }
            if (shfl && t == 0)
              for (int r = 0; r < 16; ++r) {  // 128-byte lines per warp access (coalesced layout: at most 2)
                std::set<i64> lines;
                for (int l = 0; l < 32; ++l) lines.insert(addr[l][r] >> 4);
                worst_lines = std::max(worst_lines, (int)lines.size());
              }
            host_tcm_transpose(v, gm->nswap);
            // rows: thread l of warp w now holds row 32 (w % 4) + l, columns
            // 16 h + j; the row's other half is in warp w ^ 4 (replayed too)
            cd o[32][16];
            cd vp[32][16];
            const int wp = w ^ 4;
            for (int l = 0; l < 32; ++l)
              for (int r = 0; r < 16; ++r) {
                const i64 gi = base + gm->lanes[l] + gm->rowhi[wp & 3] + ((wp >> 2) ? gm->chi : 0) + gm->clo[r];
                vp[l][r] = (gi >= 0 && gi < N) ? psi[gi] : cd(0, 0);
              }
            host_tcm_transpose(vp, gm->nswap);
            const int h = w >> 2;
            for (int l = 0; l < 32; ++l) {
              cd rowv[32];
              for (int j = 0; j < 16; ++j) {
                rowv[16 * h + j] = v[l][j];
                rowv[16 * (1 - h) + j] = vp[l][j];
              }
              for (int j = 0; j < 16; ++j) o[l][j] = block_row(U, idx, 16 * h + j, rowv);
            }
            host_tcm_transpose(o, gm->nswap);
            for (int l = 0; l < 32; ++l)
              for (int r = 0; r < 16; ++r) {
                const i64 gi = addr[l][r];
                if (gi < 0 || gi >= N) { bad = true; continue; }
                wrote[gi]++;
                out[gi] = o[l][r];
              }
          }
        }
        double err = 0, nrm = 0;
        for (i64 i = 0; i < N; ++i) {
          if (seen[i] != 1 || wrote[i] != 1) bad = true;
          err = std::max(err, std::abs(out[i] - ref[i]));
          nrm = std::max(nrm, std::abs(ref[i]));
        }
        if (shfl && worst_lines > 2) bad = true;
        if (bad || err > 1e-9 * nrm) {
          ++fails;
          printf("FAIL tensor-memory variant (%s lanes) n=%d block bits %d,%d,%d,%d,%d err=%g bad=%d lines=%d\n",
                 shfl ? "coalesced" : "strided", n, tb[0], tb[1], tb[2], tb[3], tb[4], err, (int)bad, worst_lines);
        }
        delete gm;
      }
    }
  }
  // the plan picks the measured best of the three on the 12 swept placements
  const std::vector<std::pair<std::vector<int>, int>> best = {
      {{5, 10, 15, 20, 25}, TCM_SHFL}, {{0, 10, 15, 20, 25}, TCM_SHFL}, {{4, 10, 15, 20, 25}, TCM_SHFL},
      {{3, 4, 12, 18, 24}, TCM_STRIDED}, {{0, 2, 12, 18, 24}, TCM_SHFL}, {{2, 3, 4, 15, 25}, TCM_STRIDED},
      {{0, 2, 4, 15, 25}, TCM_STRIDED}, {{0, 1, 12, 18, 24}, TCM_SHFL}, {{0, 1, 2, 15, 25}, TCM_SHFL},
      {{1, 2, 3, 4, 20}, TCM_OFF}, {{0, 1, 2, 3, 20}, TCM_OFF}, {{0, 1, 2, 3, 4}, TCM_OFF}};
  for (const auto& pb : best) {
    TcmGeom gm;
    int cb[5];
    make_geom_m(30, pb.first, true, &gm, cb);
    if (tcm_plan(pb.first) != pb.second || tcm_swaps(pb.first) != gm.nswap) {
      printf("FAIL tcm_plan on block bits %d,%d,%d,%d,%d\n", pb.first[0], pb.first[1], pb.first[2], pb.first[3],
             pb.first[4]);
      ++fails;
    }
  }
  return fails;
}

int main(int argc, char** argv) {
  if (argc > 1 && !strcmp(argv[1], "plans")) {  // tcm_plan of every 5-bit block of a 16-qubit state
    for (int m = 0; m < (1 << 16); ++m) {
      if (__builtin_popcount(m) != 5) continue;
      std::vector<int> tb;
      for (int b = 0; b < 16; ++b)
        if ((m >> b) & 1) tb.push_back(b);
      printf("%d,%d,%d,%d,%d %d\n", tb[0], tb[1], tb[2], tb[3], tb[4], tcm_plan(tb));
    }
    return 0;
  }
  std::mt19937_64 rng(5);
  std::normal_distribution<double> nd;
  int fails = 0, cases = 0, bank_fails = 0;
  for (int n = 5; n <= 16; ++n) {
    for (int trial = 0; trial < 24; ++trial) {
      std::vector<int> all(n);
      for (int i = 0; i < n; ++i) all[i] = i;
      std::shuffle(all.begin(), all.end(), rng);
      std::vector<int> tb(all.begin(), all.begin() + 5);
      if (trial == 0) tb = {4, 3, 2, 1, 0};
      if (trial == 1) tb = {n - 1, n - 2, n - 3, n - 4, n - 5};
      if (trial == 2) tb = {0, 1, 2, 3, 4};
      std::vector<zd> U(1024);
      for (auto& c : U) c = zd(nd(rng), nd(rng));
      TcGeom* geo = new TcGeom();
      int cbit[5], idx[32];
      make_geom(n, tb, geo, cbit);
      block_perm(cbit, idx);
      int t4 = 0;
      for (int b : tb) t4 += b < 4;
      const i64 N = (i64)1 << n;
      std::vector<cd> psi(N), out(N, cd(0, 0)), ref(N);
      for (auto& x : psi) x = cd(nd(rng), nd(rng));
      for (i64 i = 0; i < N; ++i) {  // the block applied directly
        int bi = 0;
        for (int jt = 0; jt < 5; ++jt) bi |= (int)((i >> tb[jt]) & 1) << (4 - jt);
        if (bi) continue;
        i64 id[32];
        for (int b = 0; b < 32; ++b) {
          id[b] = i;
          for (int jt = 0; jt < 5; ++jt)
            if ((b >> (4 - jt)) & 1) id[b] |= (i64)1 << tb[jt];
        }
        for (int r = 0; r < 32; ++r) {
          cd acc = 0;
          for (int c = 0; c < 32; ++c) acc += cd(U[r * 32 + c].real(), U[r * 32 + c].imag()) * psi[id[c]];
          ref[id[r]] = acc;
        }
      }
      const int TN = 1 << geo->nbits;
      const int nr = TN >= TC_THREADS ? TN / TC_THREADS : 1;
      const int nrows = TN >> 5;
      const i64 ntiles = (i64)1 << (n - geo->nbits);
      std::map<uint32_t, std::pair<int, int>> dec;  // A byte offset -> (row, k)
      for (int row = 0; row < TC_M; ++row)
        for (int k = 0; k < TC_K; ++k) dec[core_off(row, k, geo->a_lbo, TC_A_SBO)] = {row, k};
      std::vector<int> seen(N, 0), wrote(N, 0);
      bool bad = false;
      for (i64 t = 0; t < ntiles; ++t) {
        const i64 base = host_tile_base(t, *geo);
        std::vector<double> A(TC_M * TC_K, 0.0);
        std::set<uint32_t> used;
        for (int r = 0; r < TC_STEPS; ++r) {
          for (int tid = 0; tid < TC_THREADS; ++tid) {
            if (!(tid < TN && r < nr)) continue;
            const i64 gi = base + (tid & 127) + ((tid >> 7) ? geo->g7 : 0) + geo->ghi[r];
            if (gi < 0 || gi >= N) { bad = true; continue; }
            seen[gi]++;
            const uint32_t o = geo->aoff_lo[tid] + geo->aoff_hi[r];
            if (o + 8 > (uint32_t)TC_A_BYTES || !dec.count(o) || used.count(o)) { bad = true; continue; }
            used.insert(o);
            const auto rk = dec[o];
            A[rk.first * TC_K + rk.second] = psi[gi].real();
            A[rk.first * TC_K + rk.second + 1] = psi[gi].imag();
          }
          if (t == 0 && TN == TC_TILE)
            for (int w = 0; w < TC_THREADS / 32; ++w) {
              uint32_t off[32];
              for (int l = 0; l < 32; ++l) off[l] = geo->aoff_lo[32 * w + l] + geo->aoff_hi[r];
              if (wavefronts(off) > (t4 >= 1 ? 2 : 4)) bank_fails++;
            }
        }
        std::vector<cd> stage(TC_TILE, cd(1e300, 0));
        for (int row = 0; row < nrows; ++row)
          for (int c = 0; c < 32; ++c) {
            cd acc = 0;
            for (int k = 0; k < 32; ++k) {
              const zd u = U[idx[c] * 32 + idx[k]];
              acc += cd(u.real(), u.imag()) * cd(A[row * TC_K + 2 * k], A[row * TC_K + 2 * k + 1]);
            }
            const uint32_t si = (uint32_t)row ^ geo->scol[c];
            if (si >= (uint32_t)TC_TILE) { bad = true; continue; }
            stage[si] = acc;
          }
        if (t == 0 && TN == TC_TILE)
          for (int w = 0; w < 4; ++w)
            for (int c = 0; c < 32; ++c) {
              uint32_t off[32];
              for (int l = 0; l < 32; ++l) off[l] = 8 * ((uint32_t)(32 * w + l) ^ geo->scol[c]);
              if (wavefronts(off) > 2) bank_fails++;
            }
        for (int r = 0; r < TC_STEPS; ++r) {
          for (int tid = 0; tid < TC_THREADS; ++tid) {
            if (!(tid < TN && r < nr)) continue;
            const i64 gi = base + (tid & 127) + ((tid >> 7) ? geo->g7 : 0) + geo->ghi[r];
            if (gi < 0 || gi >= N) { bad = true; continue; }
            const uint32_t si = (uint32_t)geo->sread_lo[tid] ^ geo->sread_hi[r];
            if (si >= (uint32_t)TC_TILE) { bad = true; continue; }
            wrote[gi]++;
            out[gi] = stage[si];
          }
          if (t == 0 && TN == TC_TILE)
            for (int w = 0; w < TC_THREADS / 32; ++w) {
              uint32_t off[32];
              for (int l = 0; l < 32; ++l) off[l] = 8 * ((uint32_t)geo->sread_lo[32 * w + l] ^ geo->sread_hi[r]);
              if (wavefronts(off) > 2) bank_fails++;
            }
        }
      }
      double err = 0, nrm = 0;
      for (i64 i = 0; i < N; ++i) {
        if (seen[i] != 1 || wrote[i] != 1) bad = true;
        err = std::max(err, std::abs(out[i] - ref[i]));
        nrm = std::max(nrm, std::abs(ref[i]));
      }
      ++cases;
      if (bad || err > 1e-9 * nrm) {
        ++fails;
        printf("FAIL n=%d block bits %d,%d,%d,%d,%d err=%g bad=%d\n", n, tb[0], tb[1], tb[2], tb[3], tb[4], err,
               (int)bad);
      }
      delete geo;
    }
  }
  const int tcm_fails = check_tcm(rng);
  printf("cases %d index failures %d bank-pattern failures %d; tensor-memory variant failures %d\n", cases, fails,
         bank_fails, tcm_fails);
  return (fails || bank_fails || tcm_fails) ? 1 : 0;
}
