// Learned form kernels: descriptors, network, forces, training (see learned.h).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <stdexcept>

#include "forces.cuh"
#include "learned.h"

namespace pfmd {
namespace learned {

// ---------------------------------------------------------------------------
// model set-up and files
// ---------------------------------------------------------------------------
Model default_model(int kind, unsigned seed) {
  Model m;
  m.kind = kind;
  DescPar& d = m.d;
  d.rc_rad = kind == 0 ? 4.0f : 5.0f;
  d.rc_ang = kind == 0 ? 4.0f : 3.0f;
  const float r0 = kind == 0 ? 0.8f : 1.8f;
  const float dr = (d.rc_rad - r0) / (NR - 1);
  for (int k = 0; k < NR; ++k) {
    d.rs[k] = r0 + dr * k;
    d.eta_r[k] = 1.0f / (2.0f * dr * dr);  // Gaussians one spacing wide
  }
  d.eta_a[0] = 0.0f;
  d.eta_a[1] = kind == 0 ? 0.1f : 0.2f;
  d.bA = d.bp = d.br0 = d.bR1 = d.bR2 = 0.f;  // set from the interaction when trained
  const float z[4] = {1.f, 2.f, 4.f, 8.f};
  for (int k = 0; k < 4; ++k) d.zeta[k] = z[k];
  d.lambda[0] = 1.f;
  d.lambda[1] = -1.f;
  for (int f = 0; f < NG; ++f) {
    d.mean[f] = 0.f;
    d.inv_std[f] = 1.f;
  }
  // Glorot-uniform weights from a seeded generator, zero biases
  std::mt19937 rng(seed + 7919u * static_cast<unsigned>(kind));
  auto fill = [&](float* w, int fan_in, int fan_out, int n) {
    const float a = std::sqrt(6.f / static_cast<float>(fan_in + fan_out));
    std::uniform_real_distribution<float> U(-a, a);
    for (int i = 0; i < n; ++i) w[i] = U(rng);
  };
  fill(m.n.W1, NG, NH, NH * NG);
  fill(m.n.W2, NH, NH, NH * NH);
  fill(m.n.w3, NH, 1, NH);
  std::memset(m.n.b1, 0, sizeof(m.n.b1));
  std::memset(m.n.b2, 0, sizeof(m.n.b2));
  m.n.b3 = 0.f;
  return m;
}

// version 2: the descriptor set carries the pair baseline
static const char kMagic[8] = {'P', 'F', 'M', 'D', 'M', 'L', 'P', '2'};

void save_models(const std::string& path, const std::vector<Model>& ms) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  const int n = static_cast<int>(ms.size());
  bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(&n, sizeof(int), 1, f) == 1;
  for (const auto& m : ms)
    ok = ok && std::fwrite(&m.kind, sizeof(int), 1, f) == 1 && std::fwrite(&m.d, sizeof(DescPar), 1, f) == 1 &&
         std::fwrite(&m.n, sizeof(Net), 1, f) == 1;
  std::fclose(f);
  if (!ok) throw std::runtime_error("cannot write " + path);
}

std::vector<Model> load_models(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot open " + path);
  char mg[8];
  int n = 0;
  std::vector<Model> ms;
  bool ok = std::fread(mg, 1, 8, f) == 8 && std::memcmp(mg, kMagic, 8) == 0 && std::fread(&n, sizeof(int), 1, f) == 1 &&
            n > 0 && n < 64;
  for (int i = 0; ok && i < n; ++i) {
    Model m;
    ok = std::fread(&m.kind, sizeof(int), 1, f) == 1 && std::fread(&m.d, sizeof(DescPar), 1, f) == 1 &&
         std::fread(&m.n, sizeof(Net), 1, f) == 1;
    ms.push_back(m);
  }
  std::fclose(f);
  if (!ok) throw std::runtime_error(path + " is not a learned-potential file");
  return ms;
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void fcut_d(float r, float rc, float& f, float& df) {
  const float k = 3.14159265358979f / rc;
  float s, c;
  __sincosf(r * k, &s, &c);
  f = 0.5f * (c + 1.f);
  df = -0.5f * k * s;
}
__device__ __forceinline__ float sigm(float x) { return 1.f / (1.f + __expf(-x)); }

// Weighted sums over the 16 angular functions of one (u, v) pair at one centre:
// SA = sum w c0 A B, SdA = sum w c0 zeta lambda t^(zeta-1) B, Se = sum w c0 A B (-2 eta).
__device__ __forceinline__ void ang_sums(const DescPar& d, const float* w, float cs, float ru2, float rv2, float& SA,
                                         float& SdA, float& Se) {
  SA = SdA = Se = 0.f;
  float B[2];
#pragma unroll
  for (int ie = 0; ie < 2; ++ie) B[ie] = __expf(-d.eta_a[ie] * (ru2 + rv2));
#pragma unroll
  for (int il = 0; il < 2; ++il) {
    const float lam = d.lambda[il];
    const float t = fmaxf(1.f + lam * cs, 0.f);
    const float t2 = t * t, t4 = t2 * t2;
    const float tz[4] = {t, t2, t4, t4 * t4};       // t^zeta
    const float tzm[4] = {1.f, t, t2 * t, t4 * t2 * t};  // t^(zeta-1)
#pragma unroll
    for (int iz = 0; iz < 4; ++iz) {
      const float c0 = iz == 0 ? 1.f : (iz == 1 ? 0.5f : (iz == 2 ? 0.125f : 0.0078125f));  // 2^(1-zeta)
#pragma unroll
      for (int ie = 0; ie < 2; ++ie) {
        const float wa = w[(il * 4 + iz) * 2 + ie] * c0 * B[ie];
        SA += wa * tz[iz];
        SdA += wa * d.zeta[iz] * lam * tzm[iz];
        Se += wa * tz[iz] * (-2.f * d.eta_a[ie]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// descriptors: one thread per row
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_desc(ListDev L, const DescPar* __restrict__ Dp, Atoms A, Box B, float* G,
                                              Ctl* ctl) {
  if (ctl->stop) return;
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= L.rows) return;
  const DescPar& d = *Dp;
  float g[NG];
#pragma unroll
  for (int f = 0; f < NG; ++f) g[f] = 0.f;
  float ux[MAX_ANG], uy[MAX_ANG], uz[MAX_ANG], ur[MAX_ANG], uf[MAX_ANG];
  int na = 0;
  const int n = L.nnum[row];
  if (n > 0) {
    const int4 pi = A.posq[L.pidx[row]];
    for (int p = 0; p < n; ++p) {
      float dr[3];
      const float r2 = mi_q(pi, A.posq[ent(L, row, p)], B, dr);
      const float r = sqrtf(r2);
      if (r < d.rc_rad) {
        float fc, dfc;
        fcut_d(r, d.rc_rad, fc, dfc);
#pragma unroll
        for (int k = 0; k < NR; ++k) {
          const float t = r - d.rs[k];
          g[k] += __expf(-d.eta_r[k] * t * t) * fc;
        }
      }
      if (r < d.rc_ang) {
        if (na < MAX_ANG) {
          float fc, dfc;
          fcut_d(r, d.rc_ang, fc, dfc);
          ux[na] = dr[0];
          uy[na] = dr[1];
          uz[na] = dr[2];
          ur[na] = r;
          uf[na] = fc;
        }
        ++na;
      }
    }
    if (na > MAX_ANG) {
      set_error(ctl, ST_PARAM, EK_NONE, row + 1, na, MAX_ANG);
      na = MAX_ANG;
    }
    for (int j = 0; j < na; ++j)
      for (int k = j + 1; k < na; ++k) {
        const float cs = (ux[j] * ux[k] + uy[j] * uy[k] + uz[j] * uz[k]) / (ur[j] * ur[k]);
        const float C = uf[j] * uf[k];
        const float rr = ur[j] * ur[j] + ur[k] * ur[k];
        float Bq[2];
#pragma unroll
        for (int ie = 0; ie < 2; ++ie) Bq[ie] = __expf(-d.eta_a[ie] * rr) * C;
#pragma unroll
        for (int il = 0; il < 2; ++il) {
          const float t = fmaxf(1.f + d.lambda[il] * cs, 0.f);
          const float t2 = t * t, t4 = t2 * t2;
          const float tz[4] = {t, 0.5f * t2, 0.125f * t4, 0.0078125f * t4 * t4};
#pragma unroll
          for (int iz = 0; iz < 4; ++iz)
#pragma unroll
            for (int ie = 0; ie < 2; ++ie) g[NR + (il * 4 + iz) * 2 + ie] += tz[iz] * Bq[ie];
        }
      }
  }
  float* out = G + (size_t)row * NG;
#pragma unroll
  for (int f = 0; f < NG; ++f) out[f] = (g[f] - d.mean[f]) * d.inv_std[f];
}

void launch_desc(const ListDev& L, const DescPar* d, const Atoms& A, const Box& B, float* G, Ctl* ctl,
                 cudaStream_t s) {
  if (L.rows == 0) return;
  k_desc<<<nblk(L.rows, 128), 128, 0, s>>>(L, d, A, B, G, ctl);
  ++g_kernel_launches;
}

// ---------------------------------------------------------------------------
// network: one warp per row, weights in shared memory
// ---------------------------------------------------------------------------
struct NetSmem {
  float W1[NH * NG], b1[NH], W2[NH * NH], b2[NH], w3[NH], b3;
};

__device__ __forceinline__ void load_net(NetSmem& S, const Net* __restrict__ net) {
  const float* src = reinterpret_cast<const float*>(net);
  float* dst = reinterpret_cast<float*>(&S);
  for (int i = threadIdx.x; i < NET_FLOATS; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
}

// Forward pass of one row held in x[0..NG) (shared): z1, a1, z2 values of this
// lane's hidden units h = lane, lane + 32; returns E in every lane.
struct Fwd {
  float z1[2], z2[2], a2[2];
};
__device__ __forceinline__ float forward_row(const NetSmem& S, const float* x, float* a1s, Fwd& F) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int h = lane + 32 * q;
    float z = S.b1[h];
#pragma unroll 8
    for (int f = 0; f < NG; ++f) z += S.W1[h * NG + f] * x[f];
    F.z1[q] = z;
    a1s[h] = z * sigm(z);
  }
  __syncwarp();
  float e = 0.f;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int h = lane + 32 * q;
    float z = S.b2[h];
#pragma unroll 8
    for (int c = 0; c < NH; ++c) z += S.W2[h * NH + c] * a1s[c];
    F.z2[q] = z;
    F.a2[q] = z * sigm(z);
    e += S.w3[h] * F.a2[q];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  return e + S.b3;
}
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigm(z);
  return s * (1.f + z * (1.f - s));
}

__global__ void __launch_bounds__(256) k_mlp(int rows, const float* __restrict__ G, const DescPar* __restrict__ Dp,
                                             const Net* __restrict__ net, float* e, float* g, Ctl* ctl) {
  __shared__ NetSmem S;
  __shared__ float xs[8][NG], a1s[8][NH], e2s[8][NH], e1s[8][NH];
  if (ctl->stop) return;
  load_net(S, net);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nw = gridDim.x * 8;
  for (int row = blockIdx.x * 8 + w; row < rows; row += nw) {
    for (int f = lane; f < NG; f += 32) xs[w][f] = G[(size_t)row * NG + f];
    __syncwarp();
    Fwd F;
    const float E = forward_row(S, xs[w], a1s[w], F);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int h = lane + 32 * q;
      e2s[w][h] = S.w3[h] * dsilu(F.z2[q]);
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int c = lane + 32 * q;
      float t = 0.f;
#pragma unroll 8
      for (int h = 0; h < NH; ++h) t += S.W2[h * NH + c] * e2s[w][h];
      e1s[w][c] = t * dsilu(F.z1[q]);
    }
    __syncwarp();
    for (int f = lane; f < NG; f += 32) {
      float t = 0.f;
#pragma unroll 8
      for (int c = 0; c < NH; ++c) t += S.W1[c * NG + f] * e1s[w][c];
      g[(size_t)row * NG + f] = t * Dp->inv_std[f];
    }
    if (lane == 0) e[row] = E;
    __syncwarp();
  }
}

void launch_mlp(int rows, const float* G, const DescPar* d, const Net* net, float* e, float* g, Ctl* ctl,
                cudaStream_t s) {
  if (rows <= 0) return;
  const int grid = std::min(nblk(rows, 8), 152 * 4);
  k_mlp<<<grid, 256, 0, s>>>(rows, G, d, net, e, g, ctl);
  ++g_kernel_launches;
}

// ---------------------------------------------------------------------------
// forces: one thread per row, gathered (no atomics)
// ---------------------------------------------------------------------------
// d T / d u for the pair (u, v) at one centre, given the weighted sums.
__device__ __forceinline__ void dT_du(const float* u, float ru, const float* v, float rv, float cs, float SA, float SdA,
                                      float Se, float fu, float dfu, float fv, float out[3]) {
  const float C = fu * fv, iuv = 1.f / (ru * rv), iuu = 1.f / (ru * ru);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float dcos = v[k] * iuv - cs * u[k] * iuu;
    out[k] = SdA * C * dcos + Se * C * u[k] + SA * dfu * fv * u[k] / ru;
  }
}

// Angular terms in two passes, each triplet evaluated once.  Centre pass, one
// thread per row j: for every pair (p, k) of j's angular partners the weighted
// sums and dT/du, dT/dv give j's own force term (dT/du + dT/dv) and the legs'
// gradients, summed per partner slot into leg[p][j].  Gather pass, one thread per
// row i: radial terms, i's centre term, and -leg[q][j] for every angular
// neighbour j, q being i's slot in j's row.
__global__ void __launch_bounds__(128) k_lcenter(ListDev L, const DescPar* __restrict__ Dp,
                                                 const float* __restrict__ g, Atoms A, Box B, float4* leg,
                                                 float4* cforce, Ctl* ctl) {
  if (ctl->stop) return;
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= L.rows) return;
  const DescPar& d = *Dp;
  const int n = L.nnum[row];
  float ux[MAX_ANG], uy[MAX_ANG], uz[MAX_ANG], ur[MAX_ANG], uf[MAX_ANG], udf[MAX_ANG];
  float lx[MAX_ANG], ly[MAX_ANG], lz[MAX_ANG];
  int sl[MAX_ANG];
  int na = 0;
  float fx = 0.f, fy = 0.f, fz = 0.f;
  if (n > 0) {
    const int4 pj = A.posq[L.pidx[row]];
    for (int p = 0; p < n && na < MAX_ANG; ++p) {
      float dr[3];
      const float r = sqrtf(mi_q(pj, A.posq[ent(L, row, p)], B, dr));
      if (r < d.rc_ang) {
        fcut_d(r, d.rc_ang, uf[na], udf[na]);
        ux[na] = dr[0];
        uy[na] = dr[1];
        uz[na] = dr[2];
        ur[na] = r;
        lx[na] = ly[na] = lz[na] = 0.f;
        sl[na] = p;
        ++na;
      }
    }
    const float* gj = g + (size_t)row * NG + NR;
    for (int a = 0; a < na; ++a)
      for (int c = a + 1; c < na; ++c) {
        const float u[3] = {ux[a], uy[a], uz[a]}, v[3] = {ux[c], uy[c], uz[c]};
        const float cs = (u[0] * v[0] + u[1] * v[1] + u[2] * v[2]) / (ur[a] * ur[c]);
        float SA, SdA, Se;
        ang_sums(d, gj, cs, ur[a] * ur[a], ur[c] * ur[c], SA, SdA, Se);
        float tu[3], tv[3];
        dT_du(u, ur[a], v, ur[c], cs, SA, SdA, Se, uf[a], udf[a], uf[c], tu);
        dT_du(v, ur[c], u, ur[a], cs, SA, SdA, Se, uf[c], udf[c], uf[a], tv);
        fx += tu[0] + tv[0];
        fy += tu[1] + tv[1];
        fz += tu[2] + tv[2];
        lx[a] += tu[0];
        ly[a] += tu[1];
        lz[a] += tu[2];
        lx[c] += tv[0];
        ly[c] += tv[1];
        lz[c] += tv[2];
      }
    for (int a = 0; a < na; ++a) leg[(size_t)sl[a] * L.stride + row] = make_float4(lx[a], ly[a], lz[a], 0.f);
  }
  cforce[row] = make_float4(fx, fy, fz, 0.f);
}

// The baseline's pair function phi(r) = exp(-bp (r/br0 - 1)) fc(r) and dphi/dr,
// fc the reference's cosine switch between bR1 and bR2 (cut_off_function.f90:6-28,
// its truncated pi).
__device__ __forceinline__ void base_phi(const DescPar& d, float r, float& phi, float& dphi) {
  phi = dphi = 0.f;
  if (r >= d.bR2) return;
  const float e = __expf(-d.bp * (r / d.br0 - 1.f));
  float fc = 1.f, dfc = 0.f;
  if (r > d.bR1) {
    const float k = 3.14159265358979f / (d.bR2 - d.bR1);
    float sn, cs;
    __sincosf(k * (r - d.bR1), &sn, &cs);
    fc = 0.5f * (1.f + cs);
    dfc = -0.5f * k * sn;
  }
  phi = e * fc;
  dphi = e * (dfc - d.bp / d.br0 * fc);
}

// The model's pair terms of one list entry at distance r (separation dr, from
// the row atom to the partner): the close-contact wall and the baseline.  Adds
// the row's share of their energy to e and returns c with F_row += c dr; each
// pair sits in both atoms' rows, so c carries both rows' derivatives.
__device__ __forceinline__ float pair_terms(const DescPar& d, float rcore, float r, float& e) {
  float c = 0.f;
  if (r < rcore) {  // (k/2) (rcore - r)^2 per entry
    const float x = rcore - r;
    c -= 2.f * kCoreK * x / r;
    e += 0.5f * kCoreK * x * x;
  }
  if (d.bA > 0.f) {  // bA phi(r) per entry (the rjl repulsion is a full-row sum)
    float ph, dph;
    base_phi(d, r, ph, dph);
    c += 2.f * d.bA * dph / r;
    e += d.bA * ph;
  }
  return c;
}

__global__ void __launch_bounds__(128) k_lforce(ListDev L, const DescPar* __restrict__ Dp, const float* __restrict__ g,
                                                const float* __restrict__ erow, const float4* __restrict__ leg,
                                                const float4* __restrict__ cforce, int energy, Atoms A, Box B, Ctl* ctl,
                                                int eslot, int ekey, Epi E, float rcore) {
  if (ctl->stop) return;
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = row < L.rows;
  const DescPar& d = *Dp;
  Acc3<true> acc;
  float ei = 0.f, ep = 0.f;
  const int n = valid ? L.nnum[row] : 0;
  if (valid) {
    ei = erow[row];
    const int ai = L.pidx[row];
    const int4 pi = A.posq[ai];
    const float* gi = g + (size_t)row * NG;
    const float4 cf = cforce[row];
    acc.add(cf.x, cf.y, cf.z);
    for (int p = 0; p < n; ++p) {
      const int aj = ent(L, row, p);
      float dr[3];
      const float r = sqrtf(mi_q(pi, A.posq[aj], B, dr));
      {  // the model's pair terms besides the network: the wall and the baseline
        const float c = pair_terms(d, rcore, r, ep);
        acc.add(c * dr[0], c * dr[1], c * dr[2]);
      }
      if (r < d.rc_rad) {
        const float* gj = g + (size_t)L.row_of[aj] * NG;
        float fc, dfc;
        fcut_d(r, d.rc_rad, fc, dfc);
        float c = 0.f;
#pragma unroll
        for (int k = 0; k < NR; ++k) {
          const float t = r - d.rs[k];
          const float ex = __expf(-d.eta_r[k] * t * t);
          c += (gi[k] + gj[k]) * ex * (-2.f * d.eta_r[k] * t * fc + dfc);
        }
        const float ir = 1.f / r;
        acc.add(c * dr[0] * ir, c * dr[1] * ir, c * dr[2] * ir);
      }
      if (r < d.rc_ang) {  // i is an angular partner of j: j's centre pass holds i's leg term
        const int rj = L.row_of[aj];
        const int nj = L.nnum[rj];
        // this atom's slot in j's row: eight entries a round, their loads issued
        // together (each is its own cache line in the slot-major list)
        int slot = -1;
        for (int q0 = 0; q0 < nj && slot < 0; q0 += 8) {
          int e[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) e[u] = q0 + u < nj ? ent(L, rj, q0 + u) : -1;
#pragma unroll
          for (int u = 7; u >= 0; --u)
            if (e[u] == ai) slot = q0 + u;  // the first match of the round wins
        }
        if (slot >= 0) {
          const float4 lg = leg[(size_t)slot * L.stride + rj];
          acc.add(-lg.x, -lg.y, -lg.z);
        }
      }
    }
    finish_force(A, E, ai, acc.get(0), acc.get(1), acc.get(2));
    ei += ep;
  }
  if (energy) energy_reduce_f(ctl, eslot, ekey, ei);
}

void launch_force(const ListDev& L, const DescPar* d, const float* g, const float* e, float4* leg, float4* cforce,
                  bool energy, const Atoms& A, const Box& B, Ctl* ctl, int eslot, int ekey, cudaStream_t s,
                  const Epi& E, float rcore) {
  if (L.rows == 0) {
    if (energy) cudaMemsetAsync(&ctl->e_inter[ekey], 0, sizeof(double), s);
    return;
  }
  k_lcenter<<<nblk(L.rows, 128), 128, 0, s>>>(L, d, g, A, B, leg, cforce, ctl);
  k_lforce<<<nblk(L.rows, 128), 128, 0, s>>>(L, d, g, e, leg, cforce, energy ? 1 : 0, A, B, ctl, eslot, ekey, E,
                                             rcore);
  g_kernel_launches += 2;
}

// ---------------------------------------------------------------------------
// force matching: residuals and the descriptor vector-Jacobian product
// ---------------------------------------------------------------------------
// res[a] = 2 (f_pred - f_ref) / (3 N): dL_F/dF for L_F = sum |f_pred - f_ref|^2 / (3N)
__global__ void k_residual(int n, const double4_32a* fp, const double4_32a* fr, float4* res) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const double s = 2.0 / (3.0 * n);
  const double4_32a p = fp[a], r = fr[a];
  res[a] = make_float4((float)(s * (p.x - r.x)), (float)(s * (p.y - r.y)), (float)(s * (p.z - r.z)), 0.f);
}
void launch_residual(int n, const double4_32a* fpred, const double4_32a* fref, float4* res, cudaStream_t s) {
  if (n <= 0) return;
  k_residual<<<nblk(n, 256), 256, 0, s>>>(n, fpred, fref, res);
  ++g_kernel_launches;
}

// U[row] = inv_std * dL_F/dG[row]: for row m,
//   radial   u_k = -sum_j phi_k'(r) e_mj . (res_j - res_m)
//   angular  u_a = -sum_{j<k} (res_j - res_m) . dT_a/du + (res_k - res_m) . dT_a/dv
// which needs only m's own neighbours.
__global__ void __launch_bounds__(128) k_desc_vjp(ListDev L, const DescPar* __restrict__ Dp, Atoms A, Box B,
                                                  const float4* __restrict__ res, float* U, Ctl* ctl) {
  if (ctl->stop) return;
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= L.rows) return;
  const DescPar& d = *Dp;
  float u[NG];
#pragma unroll
  for (int f = 0; f < NG; ++f) u[f] = 0.f;
  float ux[MAX_ANG], uy[MAX_ANG], uz[MAX_ANG], ur[MAX_ANG], uf[MAX_ANG], udf[MAX_ANG];
  float qx[MAX_ANG], qy[MAX_ANG], qz[MAX_ANG];
  int na = 0;
  const int n = L.nnum[row];
  if (n > 0) {
    const int am = L.pidx[row];
    const int4 pm = A.posq[am];
    const float4 rm = res[am];
    for (int p = 0; p < n; ++p) {
      const int aj = ent(L, row, p);
      float dr[3];
      const float r = sqrtf(mi_q(pm, A.posq[aj], B, dr));
      const float4 rj = res[aj];
      const float dx = rj.x - rm.x, dy = rj.y - rm.y, dz = rj.z - rm.z;
      if (r < d.rc_rad) {
        float fc, dfc;
        fcut_d(r, d.rc_rad, fc, dfc);
        const float proj = (dr[0] * dx + dr[1] * dy + dr[2] * dz) / r;
#pragma unroll
        for (int k = 0; k < NR; ++k) {
          const float t = r - d.rs[k];
          const float ex = __expf(-d.eta_r[k] * t * t);
          u[k] -= ex * (-2.f * d.eta_r[k] * t * fc + dfc) * proj;
        }
      }
      if (r < d.rc_ang && na < MAX_ANG) {
        fcut_d(r, d.rc_ang, uf[na], udf[na]);
        ux[na] = dr[0];
        uy[na] = dr[1];
        uz[na] = dr[2];
        ur[na] = r;
        qx[na] = dx;
        qy[na] = dy;
        qz[na] = dz;
        ++na;
      }
    }
    for (int j = 0; j < na; ++j)
      for (int k = j + 1; k < na; ++k) {
        const float a[3] = {ux[j], uy[j], uz[j]}, b[3] = {ux[k], uy[k], uz[k]};
        const float ra = ur[j], rb = ur[k];
        const float cs = (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) / (ra * rb);
        // projections of the residual differences on the three vector terms
        const float qa[3] = {qx[j], qy[j], qz[j]}, qb[3] = {qx[k], qy[k], qz[k]};
        float pc = 0.f, pe = 0.f, pfa = 0.f, pfb = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float dca = b[c] / (ra * rb) - cs * a[c] / (ra * ra);
          const float dcb = a[c] / (ra * rb) - cs * b[c] / (rb * rb);
          pc += qa[c] * dca + qb[c] * dcb;
          pe += qa[c] * a[c] + qb[c] * b[c];
          pfa += qa[c] * a[c] / ra;
          pfb += qb[c] * b[c] / rb;
        }
        const float C = uf[j] * uf[k];
        const float pf = udf[j] * uf[k] * pfa + uf[j] * udf[k] * pfb;
        float Bq[2];
#pragma unroll
        for (int ie = 0; ie < 2; ++ie) Bq[ie] = __expf(-d.eta_a[ie] * (ra * ra + rb * rb));
#pragma unroll
        for (int il = 0; il < 2; ++il) {
          const float lam = d.lambda[il];
          const float t = fmaxf(1.f + lam * cs, 0.f);
          const float t2 = t * t, t4 = t2 * t2;
          const float tz[4] = {t, t2, t4, t4 * t4};
          const float tzm[4] = {1.f, t, t2 * t, t4 * t2 * t};
#pragma unroll
          for (int iz = 0; iz < 4; ++iz) {
            const float c0 = iz == 0 ? 1.f : (iz == 1 ? 0.5f : (iz == 2 ? 0.125f : 0.0078125f));
#pragma unroll
            for (int ie = 0; ie < 2; ++ie) {
              const float v = c0 * Bq[ie] *
                              (d.zeta[iz] * lam * tzm[iz] * C * pc + tz[iz] * (-2.f * d.eta_a[ie]) * C * pe + tz[iz] * pf);
              u[NR + (il * 4 + iz) * 2 + ie] -= v;
            }
          }
        }
      }
  }
  float* out = U + (size_t)row * NG;
#pragma unroll
  for (int f = 0; f < NG; ++f) out[f] = u[f] * d.inv_std[f];
}
void launch_desc_vjp(const ListDev& L, const DescPar* d, const Atoms& A, const Box& B, const float4* res, float* U,
                     Ctl* ctl, cudaStream_t s) {
  if (L.rows == 0) return;
  k_desc_vjp<<<nblk(L.rows, 128), 128, 0, s>>>(L, d, A, B, res, U, ctl);
  ++g_kernel_launches;
}

// ---------------------------------------------------------------------------
// training: per-atom energy error plus (optionally) force matching, fixed-order
// reductions, Adam
// ---------------------------------------------------------------------------
constexpr int TROWS = 32;
struct TrainSmem {
  NetSmem S;
  float x[TROWS][NG], ut[TROWS][NG];                       // normalised descriptors, force direction
  float a1[TROWS][NH], ad1[TROWS][NH];                     // a1 and its tangent
  float P1[TROWS][NH], Q1[TROWS][NH], P2[TROWS][NH], Q2[TROWS][NH], A3[TROWS][NH];
  float de[TROWS];
  double se[TROWS];
};

int train_blocks(int rows) { return (rows + TROWS - 1) / TROWS; }

__device__ __forceinline__ float d2silu(float z) {
  const float s = sigm(z);
  return s * (1.f - s) * (2.f + z * (1.f - 2.f * s));
}

// One tile of TROWS rows.  Energy term: dL_E/dE = 2 (E - t) / rows (times wE).
// Force term (U given): s = dE/dG . U, the directional derivative of the atom's
// energy along U in normalised descriptor space; its weight gradient comes from
// propagating the tangent (z1', a1', z2') forward and both paths backward.
__global__ void __launch_bounds__(256) k_train(int rows, const float* __restrict__ G, const float* __restrict__ U,
                                               const double* __restrict__ t, float wE, float wF,
                                               const Net* __restrict__ net, float* part, double* lpart) {
  extern __shared__ __align__(16) unsigned char smem[];
  TrainSmem& T = *reinterpret_cast<TrainSmem*>(smem);
  load_net(T.S, net);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int r0 = blockIdx.x * TROWS;
  const float inv_rows = 1.f / static_cast<float>(rows);
  for (int lr = w; lr < TROWS; lr += 8) {
    const int row = r0 + lr;
    if (row >= rows) {
      for (int h = lane; h < NH; h += 32)
        T.a1[lr][h] = T.ad1[lr][h] = T.P1[lr][h] = T.Q1[lr][h] = T.P2[lr][h] = T.Q2[lr][h] = T.A3[lr][h] = 0.f;
      for (int f = lane; f < NG; f += 32) T.x[lr][f] = T.ut[lr][f] = 0.f;
      if (lane == 0) {
        T.de[lr] = 0.f;
        T.se[lr] = 0.0;
      }
      continue;
    }
    for (int f = lane; f < NG; f += 32) {
      T.x[lr][f] = G[(size_t)row * NG + f];
      T.ut[lr][f] = U ? U[(size_t)row * NG + f] : 0.f;
    }
    __syncwarp();
    Fwd F;
    const float E = forward_row(T.S, T.x[lr], T.a1[lr], F);
    const double err = (double)E - t[row];
    const float de = wE * static_cast<float>(2.0 * err) * inv_rows;
    // tangent: z1' = W1 u, a1' = silu'(z1) z1'
    float zd1[2], s1[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int h = lane + 32 * q;
      float z = 0.f;
#pragma unroll 8
      for (int f = 0; f < NG; ++f) z += T.S.W1[h * NG + f] * T.ut[lr][f];
      zd1[q] = z;
      s1[q] = dsilu(F.z1[q]);
      T.ad1[lr][h] = s1[q] * z;
    }
    __syncwarp();
    // z2' = W2 a1'; energy path d2 = de w3 silu'(z2); force path beta2 = w3 silu'(z2),
    // gamma2 = w3 silu''(z2) z2'
    float b2v[2], g2v[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int h = lane + 32 * q;
      float zd2 = 0.f;
#pragma unroll 8
      for (int c = 0; c < NH; ++c) zd2 += T.S.W2[h * NH + c] * T.ad1[lr][c];
      const float s2 = dsilu(F.z2[q]);
      const float w3 = T.S.w3[h];
      b2v[q] = w3 * s2;
      g2v[q] = w3 * d2silu(F.z2[q]) * zd2;
      T.P2[lr][h] = de * w3 * s2 + wF * g2v[q];
      T.Q2[lr][h] = wF * b2v[q];
      T.A3[lr][h] = de * F.a2[q] + wF * s2 * zd2;
      // beta2 for the W2^T product below (P1 is overwritten after it)
      T.P1[lr][h] = b2v[q];
    }
    __syncwarp();
    float wb[2], wd[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int c = lane + 32 * q;
      float sb = 0.f, sd = 0.f;
#pragma unroll 8
      for (int h = 0; h < NH; ++h) {
        const float w2 = T.S.W2[h * NH + c];
        sb += w2 * T.P1[lr][h];
        sd += w2 * T.P2[lr][h];
      }
      wb[q] = sb;
      wd[q] = sd;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int c = lane + 32 * q;
      // (W2^T P2) already carries de*d2 + wF*gamma2; add the tangent's silu'' term
      T.P1[lr][c] = s1[q] * wd[q] + wF * d2silu(F.z1[q]) * zd1[q] * wb[q];
      T.Q1[lr][c] = wF * s1[q] * wb[q];
    }
    if (lane == 0) {
      T.de[lr] = de;
      T.se[lr] = err * err;
    }
    __syncwarp();
  }
  __syncthreads();
  float* out = part + (size_t)blockIdx.x * NET_FLOATS;
  const int ob1 = NH * NG, oW2 = ob1 + NH, ob2 = oW2 + NH * NH, ow3 = ob2 + NH, ob3 = ow3 + NH;
  for (int i = threadIdx.x; i < NET_FLOATS; i += blockDim.x) {
    float s = 0.f;
    if (i < ob1) {
      const int h = i / NG, f = i % NG;
      for (int r = 0; r < TROWS; ++r) s += T.P1[r][h] * T.x[r][f] + T.Q1[r][h] * T.ut[r][f];
    } else if (i < oW2) {
      const int h = i - ob1;
      for (int r = 0; r < TROWS; ++r) s += T.P1[r][h];
    } else if (i < ob2) {
      const int h = (i - oW2) / NH, c = (i - oW2) % NH;
      for (int r = 0; r < TROWS; ++r) s += T.P2[r][h] * T.a1[r][c] + T.Q2[r][h] * T.ad1[r][c];
    } else if (i < ow3) {
      const int h = i - ob2;
      for (int r = 0; r < TROWS; ++r) s += T.P2[r][h];
    } else if (i < ob3) {
      const int h = i - ow3;
      for (int r = 0; r < TROWS; ++r) s += T.A3[r][h];
    } else {
      for (int r = 0; r < TROWS; ++r) s += T.de[r];
    }
    out[i] = s;
  }
  if (threadIdx.x == 0) {
    double se = 0.0;
    for (int r = 0; r < TROWS; ++r) se += T.se[r];
    lpart[blockIdx.x] = se;
  }
}

__global__ void k_train_reduce(int blocks, int rows, const float* part, const double* lpart, float* grad, double* loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NET_FLOATS) {
    float s = 0.f;
    for (int b = 0; b < blocks; ++b) s += part[(size_t)b * NET_FLOATS + i];
    grad[i] = s;
  }
  if (i == 0) {
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += lpart[b];
    loss[0] = s;
    loss[1] = rows;
  }
}

__global__ void k_adam(float* w, const float* grad, float* m, float* v, float lr, float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NET_FLOATS) return;
  const float gi = grad[i];
  const float mi = 0.9f * m[i] + 0.1f * gi;
  const float vi = 0.999f * v[i] + 0.001f * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + 1e-8f);
}

void launch_train_grad(int rows, const float* G, const float* U, const double* target_by_row, float wE, float wF,
                       const Net* net, TrainBuf& T, cudaStream_t s) {
  const int blocks = train_blocks(rows);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sizeof(TrainSmem)));
    attr = true;
  }
  k_train<<<blocks, 256, sizeof(TrainSmem), s>>>(rows, G, U, target_by_row, wE, U ? wF : 0.f, net, T.part,
                                                 T.lpart);
  ++g_kernel_launches;
  launch_train_reduce(blocks, rows, T, s);
}

void launch_train_reduce(int blocks, int rows, TrainBuf& T, cudaStream_t s) {
  k_train_reduce<<<nblk(NET_FLOATS, 256), 256, 0, s>>>(blocks, rows, T.part, T.lpart, T.grad, T.loss);
  ++g_kernel_launches;
}

void launch_adam(Net* net, TrainBuf& T, int step, float lr, cudaStream_t s) {
  const float bc1 = 1.f - std::pow(0.9f, static_cast<float>(step));
  const float bc2 = 1.f - std::pow(0.999f, static_cast<float>(step));
  k_adam<<<nblk(NET_FLOATS, 256), 256, 0, s>>>(reinterpret_cast<float*>(net), T.grad, T.m, T.v, lr, bc1, bc2);
  ++g_kernel_launches;
}

__global__ void k_gather_rows(ListDev L, const double* eatom, double* t) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row < L.rows) t[row] = eatom[L.pidx[row]];
}
__global__ void k_core_sub(ListDev L, const DescPar* __restrict__ Dp, Atoms A, Box B, float rcore, double* t) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= L.rows) return;
  const DescPar& d = *Dp;
  const int n = L.nnum[row];
  const int4 pi = A.posq[L.pidx[row]];
  float e = 0.f;
  for (int p = 0; p < n; ++p) {
    float dr[3];
    const float r = sqrtf(mi_q(pi, A.posq[ent(L, row, p)], B, dr));
    pair_terms(d, rcore, r, e);
  }
  t[row] -= (double)e;
}
void launch_core_sub(const ListDev& L, const DescPar* d, const Atoms& A, const Box& B, float rcore, double* t,
                     cudaStream_t s) {
  if (L.rows <= 0) return;
  k_core_sub<<<nblk(L.rows, 128), 128, 0, s>>>(L, d, A, B, rcore, t);
  ++g_kernel_launches;
}
void launch_gather_rows(const ListDev& L, const double* eatom, double* t, cudaStream_t s) {
  if (L.rows == 0) return;
  k_gather_rows<<<nblk(L.rows, 256), 256, 0, s>>>(L, eatom, t);
  ++g_kernel_launches;
}

__global__ void k_force_diff(int n, const double4_32a* f, const double4_32a* fr, double* part) {
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double4_32a a = f[i], b = fr[i];
    const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    v[0] += dx * dx + dy * dy + dz * dz;
    v[1] += b.x * b.x + b.y * b.y + b.z * b.z;
  }
  block_sum<2>(v);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = v[0];
    part[2 * blockIdx.x + 1] = v[1];
  }
}
__global__ void k_force_diff_sum(int blocks, const double* part, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a = 0.0, b = 0.0;
  for (int i = 0; i < blocks; ++i) {
    a += part[2 * i];
    b += part[2 * i + 1];
  }
  out[0] = a;
  out[1] = b;
}
void launch_force_diff(int n, const double4_32a* f, const double4_32a* fref, double* part, double* out,
                       cudaStream_t s) {
  const int blocks = 256;
  k_force_diff<<<blocks, 256, 0, s>>>(n, f, fref, part);
  k_force_diff_sum<<<1, 32, 0, s>>>(blocks, part, out);
  g_kernel_launches += 2;
}

}  // namespace learned
}  // namespace pfmd
