// Periodic fluids with subcell lists: the subcell grid build, the FP64 energies, the
// grand-canonical WCA kernel and the launchers (the move kernel is in
// sadmc_cell_kernel.cuh; its WL and SAMC specialisations in sadmc_cell_wl.cu and
// sadmc_cell_samc.cu).
#include "sadmc_cell_kernel.cuh"

namespace sadmc {
cudaError_t launch_cell_move_wl(const MoveLaunch& m, const CellSys& s, int lpw, cudaStream_t st);
cudaError_t launch_cell_move_samc(const MoveLaunch& m, const CellSys& s, int lpw, cudaStream_t st);
namespace dev {

// Subcell grid of each walker (one thread per walker, atoms in index order):
// n_c = floor(L / r_cut) per axis (optcell.rs:63-73), subcell of each atom
// (optcell.rs:112-124) and the binary32 position copy.
__global__ void cell_build_kernel(const WalkerCore* cores, CellSys s, int n_walkers) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n_walkers) return;
  const int n = cores[w].n;
  const double* p = s.pos + (size_t)w * 3 * s.np;
  float4* p32 = reinterpret_cast<float4*>(s.pos32) + (size_t)w * 2 * s.np;
  int* cell_of = s.cell_of + (size_t)w * s.np;
  int* cnt = s.cell_count + (size_t)w * s.cell_cap;
  int* atoms = s.cell_atoms + (size_t)w * s.cell_cap * s.bucket;
  double L[3];
  int nc[3];
  for (int a = 0; a < 3; ++a) {
    L[a] = s.box[3 * w + a];
    nc[a] = (int)floor(L[a] / s.r_cut);
    s.ncell[3 * w + a] = nc[a];
  }
  int* status = s.build_status + w;
  *status = 0;
  if (nc[0] < 3 || nc[1] < 3 || nc[2] < 3 || nc[0] * nc[1] * nc[2] > s.cell_cap) {
    *status = ST_BAD_INPUT;
    return;
  }
  for (int c = 0; c < nc[0] * nc[1] * nc[2]; ++c) cnt[c] = 0;
  for (int i = 0; i < n; ++i) {
    const double x = p[i], y = p[s.np + i], z = p[2 * s.np + i];
    if (s.kind == SYS_WCA) put_ds<true>(p32, i, x, y, z);
    else put_ds<false>(p32, i, x, y, z);
    if (!(x >= 0.0 && x < L[0] && y >= 0.0 && y < L[1] && z >= 0.0 && z < L[2])) {
      *status = ST_BAD_INPUT;
      return;
    }
    const int cx = subcell_axis(x, L[0], nc[0]), cy = subcell_axis(y, L[1], nc[1]),
              cz = subcell_axis(z, L[2], nc[2]);
    const int c = (cx * nc[1] + cy) * nc[2] + cz;
    if (cnt[c] >= s.bucket) { *status = ST_CELL_OVERFLOW; return; }
    atoms[(size_t)c * s.bucket + cnt[c]] = i;
    cnt[c] += 1;
    cell_of[i] = c;
  }
}

// compute_energy: WCA (wca.rs:222-230) and square well (optsquare.rs:176-186) in FP64
// over the same candidate images.  One warp per walker.
template <int KIND>
__global__ void cell_energy_kernel(const WalkerCore* cores, CellSys s, int n_walkers, double* out) {
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (w >= n_walkers) return;
  const int n = cores[w].n;
  const double* p = s.pos + (size_t)w * 3 * s.np;
  const int* cell_of = s.cell_of + (size_t)w * s.np;
  const int* cnt = s.cell_count + (size_t)w * s.cell_cap;
  const int* atoms = s.cell_atoms + (size_t)w * s.cell_cap * s.bucket;
  double L[3];
  int nc[3];
  for (int a = 0; a < 3; ++a) { L[a] = s.box[3 * w + a]; nc[a] = s.ncell[3 * w + a]; }
  const double rc2 = s.r_cut * s.r_cut;
  double e = 0.0;
  long long contacts = 0;
  for (int i = lane; i < n; i += 32) {
    const double ix = p[i], iy = p[s.np + i], iz = p[2 * s.np + i];
    const int ci = cell_of[i];
    const int cx = ci / (nc[1] * nc[2]), cy = (ci / nc[2]) % nc[1], cz = ci % nc[2];
    for (int k0 = 0; k0 < 27; ++k0) {
      const int dx = k0 / 9 - 1, dy = (k0 / 3) % 3 - 1, dz = k0 % 3 - 1;
      int ux = cx + dx, uy = cy + dy, uz = cz + dz, ox = 0, oy = 0, oz = 0;
      if (ux < 0) { ux += nc[0]; ox = 1; } else if (ux >= nc[0]) { ux -= nc[0]; ox = -1; }
      if (uy < 0) { uy += nc[1]; oy = 1; } else if (uy >= nc[1]) { uy -= nc[1]; oy = -1; }
      if (uz < 0) { uz += nc[2]; oz = 1; } else if (uz >= nc[2]) { uz -= nc[2]; oz = -1; }
      const int c = (ux * nc[1] + uy) * nc[2] + uz;
      for (int q = 0; q < cnt[c]; ++q) {
        const int j = atoms[(size_t)c * s.bucket + q];
        if (j == i) continue;
        // (r1 - r2) with r2 the image of j (optcell.rs:82-89)
        const double bx = ix - (p[j] - (double)ox * L[0]);
        const double by = iy - (p[s.np + j] - (double)oy * L[1]);
        const double bz = iz - (p[2 * s.np + j] - (double)oz * L[2]);
        const double d2 = bx * bx + by * by + bz * bz;
        if (KIND == SYS_SW) { if (d2 < rc2) ++contacts; }
        else e += wca_v64(d2, rc2);
      }
    }
  }
  if (KIND == SYS_SW) {
    for (int o = 16; o > 0; o >>= 1) contacts += __shfl_xor_sync(0xffffffffu, contacts, o);
    if (lane == 0) out[w] = -(double)contacts * 0.5;
  } else {
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if (lane == 0) out[w] = e * 0.5;
  }
}

// Grand-canonical WCA fluid with the energy-number method (src/mc/energy_number.rs,
// wca.rs:307-323): translations (wca.rs:342-353), adds at a uniform point of the box
// (add_atom_at, wca.rs:105-116; optcell.rs:126-130) and removals of a uniform atom
// (remove_atom_number, wca.rs:151-163; optcell.rs:177-193: swap_remove, the last atom
// takes the removed index).  LPW lanes per walker over the subcell buckets (32 by
// default: a batch of a few hundred walkers needs the warps).
template <int LPW>
__global__ void __launch_bounds__(128) wca_grand_kernel(GrandLaunch m) {
  constexpr int WPW = 32 / LPW;
  const int group = (threadIdx.x & 31) / LPW, glane = (threadIdx.x & 31) % LPW;
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * WPW + group;
  // every collective below is over the walker's own group: a group past the last walker
  // leaves without disturbing the others
  if (w >= m.n_walkers) return;
  const unsigned gmask = group_mask<LPW>(group);
  GrandBook<LPW> bk;
  bk.load(m, w, glane, gmask);
  CellWalker cw;
  cw.np = m.np;
  cw.bucket = m.bucket;
  cw.p = m.pos64 + (size_t)w * 3 * m.np;
  cw.p32 = reinterpret_cast<float4*>(m.pos32) + (size_t)w * 2 * m.np;
  cw.cell_of = m.cell_of + (size_t)w * m.np;
  cw.cnt = m.cell_count + (size_t)w * m.cell_cap;
  cw.atoms = m.cell_atoms + (size_t)w * m.cell_cap * m.bucket;
  for (int a = 0; a < 3; ++a) {
    cw.L[a] = m.box[a];
    cw.L32[a] = (float)m.box[a];
    cw.Ll32[a] = (float)(m.box[a] - (double)cw.L32[a]);
    cw.nc[a] = m.nc[a];
  }
  const double wsqr = m.r_cut * m.r_cut;
  const float wsqr32 = (float)wsqr;
  auto cell_xyz = [&](int c, int& x, int& y, int& z) {
    x = c / (cw.nc[1] * cw.nc[2]);
    y = (c / cw.nc[2]) % cw.nc[1];
    z = c % cw.nc[2];
  };
  // binary32 energy of a query point against the candidates of its 27 subcells
  auto near32 = [&](double qx, double qy, double qz, int c, int skip) -> float {
    int cx, cy, cz;
    cell_xyz(c, cx, cy, cz);
    int cn = 0;
    bool ov = false;
    float e = 0.0f;
    const Query q = make_query<true>(qx, qy, qz);
    // one bucket per lane: the grand fluids are sparse (mostly empty subcells), where
    // spreading the candidates over the group costs more than it saves
    for (int k = glane; k < 27; k += LPW)
      CellOps<LPW, SYS_WCA>::scan(cw, k, cx, cy, cz, q, skip, wsqr, wsqr32, true, cn, ov, e);
    return group_sum<LPW>(e, gmask);
  };
  const double sc = m.translation_scale;
  Every resum;
  resum.init(bk.c.moves, m.resum_interval > 0 ? (uint64_t)m.resum_interval : 0);
  for (uint64_t it = 0; it < m.n_moves; ++it) {
    bk.c.moves += 1;
    const uint64_t t = bk.c.moves;
    const GrandDraws d = draws_grand(m.seed, (uint32_t)w, t);
    const double E1 = bk.c.E;
    const int N1 = bk.c.N;
    int kind_move = -1, which = 0, N2 = N1, new_c = 0;
    double tx = 0, ty = 0, tz = 0;
    float de = 0.0f;
    const bool translation = bk.choose(d);
    if (translation) {
      if (N1 > 0) {  // plan_move: put_in_cell(from + g * scale)
        which = (int)mulhi_range(d.pick, (uint32_t)N1);
        const double fx = cw.p[which], fy = cw.p[cw.np + which], fz = cw.p[2 * cw.np + which];
        bool bad = false;
        tx = wrap_axis(fx + (double)d.g0 * sc, cw.L[0], &bad);
        ty = wrap_axis(fy + (double)d.g1 * sc, cw.L[1], &bad);
        tz = wrap_axis(fz + (double)d.g2 * sc, cw.L[2], &bad);
        new_c = cw.cell_index(subcell_axis(tx, cw.L[0], cw.nc[0]), subcell_axis(ty, cw.L[1], cw.nc[1]),
                              subcell_axis(tz, cw.L[2], cw.nc[2]));
        const int old_c = cw.cell_of[which];
        de = near32(tx, ty, tz, new_c, which) - near32(fx, fy, fz, old_c, which);
        if (!bad && !(new_c != old_c && min(cw.cnt[new_c], cw.bucket) >= cw.bucket)) kind_move = 0;
        else if (!bad) bk.c.status |= ST_CELL_OVERFLOW;
      }
    } else if (d.add_bit == 0) {
      if (!(m.has_max_N && N1 == m.max_N) && N1 < cw.np) {
        // a uniform point of the box (words of add candidate 0), then put_in_cell
        const uint32_t k0 = (uint32_t)w, k1 = (uint32_t)m.seed, shi = (uint32_t)(m.seed >> 32);
        const Philox4 D = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 8u, shi}, k0, k1);
        const Philox4 Q = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 9u, shi}, k0, k1);
        const double s53 = 1.0 / 9007199254740992.0;
        bool bad = false;
        tx = wrap_axis(cw.L[0] * ((double)u53_bits(D.x, D.y) * s53), cw.L[0], &bad);
        ty = wrap_axis(cw.L[1] * ((double)u53_bits(D.z, D.w) * s53), cw.L[1], &bad);
        tz = wrap_axis(cw.L[2] * ((double)u53_bits(Q.x, Q.y) * s53), cw.L[2], &bad);
        new_c = cw.cell_index(subcell_axis(tx, cw.L[0], cw.nc[0]), subcell_axis(ty, cw.L[1], cw.nc[1]),
                              subcell_axis(tz, cw.L[2], cw.nc[2]));
        de = near32(tx, ty, tz, new_c, -1);
        if (min(cw.cnt[new_c], cw.bucket) < cw.bucket) {
          kind_move = 1;
          N2 = N1 + 1;
        } else {
          bk.c.status |= ST_CELL_OVERFLOW;
        }
      }
    } else if (N1 > 0) {
      which = (int)mulhi_range(d.pick, (uint32_t)N1);
      de = -near32(cw.p[which], cw.p[cw.np + which], cw.p[2 * cw.np + which], cw.cell_of[which], which);
      kind_move = 2;
      N2 = N1 - 1;
    }
    const bool possible = kind_move >= 0 && fabsf(de) <= 3.0e38f;
    if (m.trace && glane == 0 && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap) {
      TraceRec r;
      r.e1 = E1;
      r.e2 = possible ? E1 + (double)de : __longlong_as_double(0x7ff8000000000000ll);
      m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)] = r;
    }
    if (possible && bk.decide(m, E1, N1, E1 + (double)de, N2, translation, d.u53)) {
      // ConfirmSystem::confirm (wca.rs:276-301) on the buckets
      if (kind_move == 0 || kind_move == 2) {
        // take `which` out of its bucket (kept for a move within the same subcell)
        const int oc = cw.cell_of[which];
        if (kind_move == 2 || new_c != oc) {
          int* lo = cw.atoms + (size_t)oc * cw.bucket;
          const int mo = min(cw.cnt[oc], cw.bucket);
          int pos = -1;
          for (int k = glane; k < mo; k += LPW)
            if (lo[k] == which) pos = k;
#pragma unroll
          for (int o = LPW / 2; o > 0; o >>= 1) {
            const int x = __shfl_xor_sync(gmask, pos, o, LPW);
            pos = x > pos ? x : pos;
          }
          __syncwarp(gmask);
          if (glane == 0 && pos >= 0) {
            lo[pos] = lo[mo - 1];
            cw.cnt[oc] = mo - 1;
          }
          __syncwarp(gmask);
        }
      }
      if (kind_move == 0 || kind_move == 1) {
        const int a = kind_move == 0 ? which : N1;
        const int oc = kind_move == 0 ? cw.cell_of[which] : -1;
        if (glane == 0) {
          if (kind_move == 1 || new_c != oc) {
            const int cnt = cw.cnt[new_c];
            cw.atoms[(size_t)new_c * cw.bucket + cnt] = a;
            cw.cnt[new_c] = cnt + 1;
          }
          cw.cell_of[a] = new_c;
          cw.p[a] = tx; cw.p[cw.np + a] = ty; cw.p[2 * cw.np + a] = tz;
          put_ds<true>(cw.p32, a, tx, ty, tz);
        }
      } else if (which != N1 - 1) {
        // swap_remove: atom N1 - 1 takes index `which` (rename_neighbor, optcell.rs:419)
        const int last = N1 - 1, lc = cw.cell_of[last];
        int* ll = cw.atoms + (size_t)lc * cw.bucket;
        const int ml = min(cw.cnt[lc], cw.bucket);
        int pos = -1;
        for (int k = glane; k < ml; k += LPW)
          if (ll[k] == last) pos = k;
#pragma unroll
        for (int o = LPW / 2; o > 0; o >>= 1) {
          const int x = __shfl_xor_sync(gmask, pos, o, LPW);
          pos = x > pos ? x : pos;
        }
        __syncwarp(gmask);
        if (glane == 0) {
          if (pos >= 0) ll[pos] = which;
          cw.cell_of[which] = lc;
          cw.p[which] = cw.p[last];
          cw.p[cw.np + which] = cw.p[cw.np + last];
          cw.p[2 * cw.np + which] = cw.p[2 * cw.np + last];
          cw.p32[2 * which] = cw.p32[2 * last];
          cw.p32[2 * which + 1] = cw.p32[2 * last + 1];
        }
      }
      __syncwarp(gmask);
    }
    bk.finish(m, t, E1, N1);
    if (resum.tick()) {
      double e = 0.0;
      const int n = bk.c.N;
      for (int i = glane; i < n; i += LPW)
        e += cw.pair_sum64(i, [&](double r2) { return wca_v64(r2, wsqr); });
      bk.resummed(m, group_sum<LPW>(e, gmask) * 0.5);
    }
  }
  bk.store(m.cores, w);
}

}  // namespace dev

cudaError_t launch_cell_move(const MoveLaunch& m, const CellSys& s, int lpw, cudaStream_t st) {
  if (m.method == M_WL) return launch_cell_move_wl(m, s, lpw, st);
  if (m.method == M_SAMC) return launch_cell_move_samc(m, s, lpw, st);
  SADMC_CELL_ALL_SHAPES(dev::FAM_ANY)
  return cudaErrorInvalidConfiguration;
}

cudaError_t launch_cell_build(const WalkerCore* cores, const CellSys& s, int n_walkers,
                              cudaStream_t st) {
  dev::cell_build_kernel<<<(n_walkers + 127) / 128, 128, 0, st>>>(cores, s, n_walkers);
  return cudaGetLastError();
}

cudaError_t launch_cell_energy(const WalkerCore* cores, const CellSys& s, int n_walkers,
                               double* out, cudaStream_t st) {
  const int blocks = (n_walkers * 32 + 127) / 128;
  if (s.kind == SYS_SW) dev::cell_energy_kernel<SYS_SW><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out);
  else dev::cell_energy_kernel<SYS_WCA><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out);
  return cudaGetLastError();
}

}  // namespace sadmc

namespace sadmc {
cudaError_t launch_wca_grand_move(const GrandLaunch& m, cudaStream_t st) {
  const int lpw = m.lanes == 8 || m.lanes == 16 ? m.lanes : 32;
  const int warps = (m.n_walkers + (32 / lpw) - 1) / (32 / lpw);
  if (lpw == 8) dev::wca_grand_kernel<8><<<(warps + 3) / 4, 128, 0, st>>>(m);
  else if (lpw == 16) dev::wca_grand_kernel<16><<<(warps + 3) / 4, 128, 0, st>>>(m);
  else dev::wca_grand_kernel<32><<<(warps + 3) / 4, 128, 0, st>>>(m);
  return cudaGetLastError();
}
}  // namespace sadmc

