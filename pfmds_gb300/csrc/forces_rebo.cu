// rebosc: the REBO-type solid-carbon potential of REBOsolidcarbon.f90:27-92.  The
// reference has only its energy and takes the forces by central differences of
// it (calculate_forces_numerically, md_interactions.f90:273-310: dx = 1e-6 A on a
// list truncated to third neighbours, six energy evaluations per atom).  Here the
// forces are the analytic gradient of the same energy.
//
// Over bonds i < j (group order) with r = |r_ij| < R2:
//   E = sum fc(r) [ (1 + Q/r) A e^{-alpha r} - bbar_ij V_A(r) ],   V_A = sum_k B_k e^{-beta_k r}
//   bbar_ij = (bsp_ij + bsp_ji)/2 + bdh_ij
//   bsp_ij  = (1 + S_ij)^{-1/2},  S_ij = sum_{k in N(i)\j, r_ik < R2} fc(r_ik) G(cos theta_jik)
//   bdh_ij  = T sum_{k in N(i)\j, r_ik < R2} sum_{l in N(j)\i, r_jl < R2} fc(r_ik) fc(r_jl) (1 - D^2/(X Y))
// with G the quintic g1 + g2 c + ... + g6 c^5, and for a = r_ij, b = r_ik, c = r_jl:
// D = (a.a)(b.c) - (a.b)(a.c) = (a x b).(a x c), X = |a x b|^2, Y = |a x c|^2, so
// 1 - D^2/(X Y) is the squared sine of the dihedral angle k-i-j-l.
//
// Pass 1 (one thread per row i): per list slot bsp, its derivative factor
// dbsp/dS = -(1+S)^{-3/2}/2 and, for j > i, bdh.  Pass 2 (one thread per row m):
// the force on atom m gathered over every bond whose energy depends on m's
// position -- the bonds (a, b) with a a neighbour of m and b a neighbour of a,
// each taken once -- and, at energy steps, the energies of m's bonds to higher
// rows.  No atomics, so runs repeat bit for bit.  FP64 in both forms.  Requires
// g1 == g2: a partner's row is row_of[atom].
#include "forces.cuh"

namespace pfmd {

namespace {

__device__ __forceinline__ void gpoly(const REBOPar& P, double c, double& G, double& dG) {
  G = P.g[0] + c * (P.g[1] + c * (P.g[2] + c * (P.g[3] + c * (P.g[4] + c * P.g[5]))));
  dG = P.g[1] + c * (2.0 * P.g[2] + c * (3.0 * P.g[3] + c * (4.0 * P.g[4] + c * 5.0 * P.g[5])));
}

__device__ __forceinline__ double rdist(const Atoms& A, const Box& B, int from, int to, double d[3]) {
  return sqrt(mi_exact(A.pos[from], A.pos[to], B, d));
}

__device__ __forceinline__ int slot_of(const ListDev& L, int row, int atom) {
  const int n = L.nnum[row];
  int q = 0;
  for (; q < n; ++q)
    if (ent(L, row, q) == atom) break;
  return q < n ? q : -1;
}

// d S_cp / d x_m of the angle sum at centre row c for its slot e (partner atom ap,
// vector a = r_{c,ap}, length r), added to g with weight w.
__device__ void angle_grad(const ListDev& L, const REBOPar& P, const Atoms& A, const Box& B, int c, int e, int ac,
                           int ap, const double a[3], double r, int am, double w, double g[3]) {
  const int n = L.nnum[c];
  const bool mc = am == ac, mp = am == ap;
  for (int k = 0; k < n; ++k) {
    if (k == e) continue;
    const int ak = ent(L, c, k);
    if (!(mc || mp || ak == am)) continue;
    double b[3];
    const double rk = rdist(A, B, ac, ak, b);
    if (!(rk < P.R2)) continue;
    double fk, dfk;  // fc and fc'/r
    fdfcut_cos(rk, P.R1, P.R2, fk, dfk);
    const double cs = (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) / (r * rk);
    double G, dG;
    gpoly(P, cs, G, dG);
    for (int d = 0; d < 3; ++d) {
      const double ga = fk * dG * (b[d] / (r * rk) - cs * a[d] / (r * r));
      const double gb = dfk * b[d] * G + fk * dG * (a[d] / (r * rk) - cs * b[d] / (rk * rk));
      double v = 0.0;
      if (mp) v += ga;
      if (ak == am) v += gb;
      if (mc) v -= ga + gb;
      g[d] += w * v;
    }
  }
}

// d/d x_m of the dihedral double sum of bond x->y (x's slot p, y's atom ay, a = r_xy),
// added to g with weight w.
__device__ void dihedral_grad(const ListDev& L, const REBOPar& P, const Atoms& A, const Box& B, int x, int p,
                              int y, int ax, int ay, const double a[3], double r, int am, double w, double g[3]) {
  const int nx = L.nnum[x], ny = L.nnum[y];
  const bool mx = am == ax, my = am == ay;
  const double aa = r * r;
  for (int k = 0; k < nx; ++k) {
    if (k == p) continue;
    const int ak = ent(L, x, k);
    double b[3];
    const double rk = rdist(A, B, ax, ak, b);
    if (!(rk < P.R2)) continue;
    double fk, dfk;
    fdfcut_cos(rk, P.R1, P.R2, fk, dfk);
    const double bb = rk * rk, ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    const double X = aa * bb - ab * ab;
    for (int l = 0; l < ny; ++l) {
      const int al = ent(L, y, l);
      if (al == ax) continue;
      if (!(mx || my || ak == am || al == am)) continue;
      double c[3];
      const double rl = rdist(A, B, ay, al, c);
      if (!(rl < P.R2)) continue;
      double fl, dfl;
      fdfcut_cos(rl, P.R1, P.R2, fl, dfl);
      const double cc = rl * rl, ac = a[0] * c[0] + a[1] * c[1] + a[2] * c[2];
      const double bc = b[0] * c[0] + b[1] * c[1] + b[2] * c[2];
      const double Y = aa * cc - ac * ac, D = aa * bc - ab * ac;
      const double s = D * D / (X * Y), u = 2.0 * D / (X * Y), vX = s / X, vY = s / Y;
      const double ff = fk * fl, one_s = 1.0 - s;
      for (int d = 0; d < 3; ++d) {
        const double dsa = u * (2.0 * a[d] * bc - b[d] * ac - c[d] * ab) - vX * (2.0 * a[d] * bb - 2.0 * ab * b[d]) -
                           vY * (2.0 * a[d] * cc - 2.0 * ac * c[d]);
        const double dsb = u * (aa * c[d] - ac * a[d]) - vX * (2.0 * aa * b[d] - 2.0 * ab * a[d]);
        const double dsc = u * (aa * b[d] - ab * a[d]) - vY * (2.0 * aa * c[d] - 2.0 * ac * a[d]);
        const double ta = -ff * dsa;
        const double tb = dfk * b[d] * fl * one_s - ff * dsb;
        const double tc = fk * dfl * c[d] * one_s - ff * dsc;
        double v = 0.0;
        if (my) v += ta - tc;
        if (mx) v -= ta + tb;
        if (ak == am) v += tb;
        if (al == am) v += tc;
        g[d] += w * v;
      }
    }
  }
}

// The bond of rows x < y (x's slot p, y's slot q of x, -1 if absent): adds
// dE_xy/dx_m to g; returns E_xy.
__device__ double bond(const ListDev& L, const REBOPar& P, const Atoms& A, const Box& B, const double* S3,
                       size_t slab, int x, int p, int y, int q, int am, double g[3]) {
  const int ax = L.pidx[x], ay = L.pidx[y];
  double a[3];
  const double r = rdist(A, B, ax, ay, a);
  if (!(r < P.R2)) return 0.0;
  double fc, dfc;
  fdfcut_cos(r, P.R1, P.R2, fc, dfc);
  const double fp = dfc * r;
  const double ea = exp(-P.alpha * r);
  const double VR = (1.0 + P.Q / r) * P.A * ea;
  const double dVR = -P.Q / (r * r) * P.A * ea - P.alpha * VR;
  double VA = 0.0, dVA = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double t = P.B[k] * exp(-P.beta[k] * r);
    VA += t;
    dVA -= P.beta[k] * t;
  }
  const double W = fc * VA, dW = fp * VA + fc * dVA;
  const size_t sx = (size_t)p * L.stride + x;
  const double bsx = S3[sx], dbx = S3[slab + sx], bdh = S3[2 * slab + sx];
  double bsy = 0.0, dby = 0.0;
  if (q >= 0) {
    const size_t sy = (size_t)q * L.stride + y;
    bsy = S3[sy];
    dby = S3[slab + sy];
  }
  const double bbar = 0.5 * (bsx + bsy) + bdh;
  if (am == ax || am == ay) {
    const double gr = (fp * VR + fc * dVR - dW * bbar) / r;
    const double sg = am == ay ? 1.0 : -1.0;
    for (int d = 0; d < 3; ++d) g[d] += sg * gr * a[d];
  }
  angle_grad(L, P, A, B, x, p, ax, ay, a, r, am, -0.5 * W * dbx, g);
  if (q >= 0) {
    double ayx[3];
    const double ry = rdist(A, B, ay, ax, ayx);  // y's own view of the bond
    angle_grad(L, P, A, B, y, q, ay, ax, ayx, ry, am, -0.5 * W * dby, g);
  }
  dihedral_grad(L, P, A, B, x, p, y, ax, ay, a, r, am, -W * P.T, g);
  return fc * VR - bbar * W;
}

}  // namespace

__global__ void __launch_bounds__(128) k_rebo_bond(ListDev L, REBOPar P, Atoms A, Box B, double* S3, Ctl* ctl) {
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.rows) return;
  const int n = L.nnum[i];
  const int ai = L.pidx[i];
  const size_t slab = (size_t)L.nmax * L.stride;
  for (int p = 0; p < n; ++p) {
    const int aj = ent(L, i, p);
    double a[3];
    const double r = rdist(A, B, ai, aj, a);
    double bsp = 0.0, dbs = 0.0, bdh = 0.0;
    if (r < P.R2) {
      const int j = L.row_of[aj];
      const bool up = j > i;
      const int nj = up ? L.nnum[j] : 0;
      double S = 0.0;
      for (int q = 0; q < n; ++q) {
        if (q == p) continue;
        const int ak = ent(L, i, q);
        double b[3];
        const double rq = rdist(A, B, ai, ak, b);
        if (!(rq < P.R2)) continue;
        const double fq = fcut_cos(rq, P.R1, P.R2);
        const double cs = (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) / (r * rq);
        double G, dG;
        gpoly(P, cs, G, dG);
        S += fq * G;
        for (int l = 0; l < nj; ++l) {
          const int al = ent(L, j, l);
          if (al == ai) continue;
          double c[3];
          const double rl = rdist(A, B, aj, al, c);
          if (!(rl < P.R2)) continue;
          const double aa = r * r, ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
          const double ac = a[0] * c[0] + a[1] * c[1] + a[2] * c[2], bc = b[0] * c[0] + b[1] * c[1] + b[2] * c[2];
          const double D = aa * bc - ab * ac;
          bdh += fq * fcut_cos(rl, P.R1, P.R2) * (1.0 - D * D / (aa * rq * rq - ab * ab) / (aa * rl * rl - ac * ac));
        }
      }
      const double x = 1.0 + S;
      bsp = 1.0 / sqrt(x);
      dbs = -0.5 * bsp / x;
      bdh = P.T * bdh;
    }
    const size_t s = (size_t)p * L.stride + i;
    S3[s] = bsp;
    S3[slab + s] = dbs;
    S3[2 * slab + s] = bdh;
  }
}

template <bool ENERGY>
__global__ void __launch_bounds__(128) k_rebo_force(ListDev L, REBOPar P, Atoms A, Box B, const double* S3, Ctl* ctl,
                                                    int eslot, int ekey, Epi E) {
  if (ctl->stop) return;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  double erow = 0.0;
  if (m < L.rows && (L.nnum[m] > 0 || E.store || E.kick)) {
    const int nm = L.nnum[m];
    const int am = L.pidx[m];
    const size_t slab = (size_t)L.nmax * L.stride;
    double g[3] = {0.0, 0.0, 0.0};
    double eh = 0.0;
    for (int s = 0; s < nm; ++s) {
      const int aa = ent(L, m, s);
      const int ra = L.row_of[aa];
      const int na = L.nnum[ra];
      for (int t = 0; t < na; ++t) {
        const int ab = ent(L, ra, t);
        const int rb = L.row_of[ab];
        // a bond between two neighbours of m is met from both ends: keep the lower row's
        if (ab != am && ra > rb && slot_of(L, m, ab) >= 0) continue;
        double e;
        if (ra < rb)
          e = bond(L, P, A, B, S3, slab, ra, t, rb, slot_of(L, rb, aa), am, g);
        else
          e = bond(L, P, A, B, S3, slab, rb, slot_of(L, rb, aa), ra, t, am, g);
        if (ab == am) {  // one of m's own bonds
          if (ENERGY && m < ra) erow += e;
          eh += 0.5 * e;
        }
      }
    }
    finish_force(A, E, am, -g[0], -g[1], -g[2]);
    if (ENERGY && E.eatom) E.eatom[am] = eh;
  }
  if (ENERGY) energy_reduce(ctl, eslot, ekey, erow);
}

void launch_rebo(bool energy, const ListDev& L, const REBOPar& P, const Atoms& A, const Box& B, double* S3, Ctl* ctl,
                 int eslot, int ekey, cudaStream_t s, int parts, const Epi& E) {
  if (L.rows == 0) {
    if (energy && (parts & 2)) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  const int g = nblk(L.rows, 128);
  if (parts & 1) {
    k_rebo_bond<<<g, 128, 0, s>>>(L, P, A, B, S3, ctl);
    ++g_kernel_launches;
  }
  if (parts & 2) {
    if (energy)
      k_rebo_force<true><<<g, 128, 0, s>>>(L, P, A, B, S3, ctl, eslot, ekey, E);
    else
      k_rebo_force<false><<<g, 128, 0, s>>>(L, P, A, B, S3, ctl, eslot, ekey, E);
    ++g_kernel_launches;
  }
}

}  // namespace pfmd
