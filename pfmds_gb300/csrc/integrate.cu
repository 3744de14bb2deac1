// Integration, thermostat, molecular statics and the per-step control kernel.
//
// Reference: md_integrators.f90 (velocity Verlet :7-97, molecular statics :99-145,
// zero_forces :147, Nose-Hoover chain :165-260), md_general.f90 (kinetic energy,
// temperature, centre-of-mass, zero_momentum, check_positions,
// invert_z_velocities, change_particle_group_N) and the step order of
// md_simulation.f90:114-243.
//
// Kernels walk group index arrays like the reference; group sizes come from
// Ctl::group_n.  The plain form keeps the reference's operation order for the
// kick (f/m/mass_coef*dt/2) with round-to-nearest intrinsics; the precision form
// multiplies by a per-atom 1/(m*mass_coef) to keep FP64 divides off the step.
// Reductions are deterministic: block partials summed in block order by the
// last block, which also performs the scalar updates (chain, temperature).
#include "forces.cuh"

namespace pfmd {

__constant__ double c_mass_coef = 1.6605389217 / 1.6021765654 * 100.0;  // md_integrators.f90:62
__constant__ double c_kt_a_degree = 1.3806488 / 1.6021765654 * 1e-4;    // md_general.f90:304

static constexpr int kRedBlocks = 592;  // 4 x 148-152 SMs, fixed so sums are reproducible
static constexpr int kRedThreads = 256;

struct Changes {
  int n;
  ChangeSpec c[8];
};

// change_particle_group_N (md_general.f90:82-95), check_positions' verdict and the
// nvms exit test (md_simulation.f90:142-147, 158).
__global__ void k_step_begin(int phase, Changes ch, int nvms, double ms_de, Ctl* ctl) {
  if (ctl->stop) return;
  if (phase == 0 || phase == 2) {
    const long long s = ctl->md_step + 1;
    ctl->md_step = s;
    for (int k = 0; k < ch.n; ++k) {
      const ChangeSpec& c = ch.c[k];
      int n = ctl->group_n[c.to];
      if (s <= c.ts1) {
        n = ctl->group_n[c.from];
        if (s == c.ts1) n = n + 1;
      } else if (s < c.ts2 && (s - c.ts1) % c.frec == 0) {
        n = n + 1;
      }
      if (n > c.to_cap) n = c.to_cap;
      ctl->group_n[c.to] = n;
    }
    if (oob_pending(ctl)) {
      set_error(ctl, ST_OUT_OF_CELL, EK_OOB, ctl->oob_atom + 1, 0, 0);
      return;
    }
  }
  if (phase == 1 || phase == 2) {
    if (nvms && ctl->md_step != 0 && fabs(ctl->pe_last - ctl->pe_prev) <= ms_de) {
      ctl->converged = 1;
      ctl->err_step = ctl->md_step;
      ctl->stop = 1;
      return;
    }
    ctl->pe_prev = ctl->pe_last;
  }
}

__device__ __forceinline__ void flag_oob(Ctl* ctl, int i) {
  atomicMin(&ctl->oob_atom, i);
  ctl->pending_oob = 1;
}

__global__ void k_check_all(Atoms A, Box B, Ctl* ctl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.N) return;
  const double4_32a p = A.pos[i];
  if (out_of_cell(p.x, B.Ltol[0]) || out_of_cell(p.y, B.Ltol[1]) || out_of_cell(p.z, B.Ltol[2])) flag_oob(ctl, i);
}

// invert_z_velocities(atoms, 0.8*Lz, 0.9*Lz), md_general.f90:382-398
__global__ void k_invert_z(Atoms A, Box B, Ctl* ctl) {
  if (ctl->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.N) return;
  const double lo = 0.8 * B.L[2], hi = 0.9 * B.L[2];
  const double z = A.pos[i].z;
  double4_32a v = A.vel[i];
  if ((z > lo && z < (lo + hi) / 2 && v.z > 0.0) || (z < hi && z > (lo + hi) / 2 && v.z < 0.0)) {
    v.z = -v.z;
    A.vel[i] = v;
  }
}

// v = v + f/m/mass_coef*ts(2), in the reference's order (md_integrators.f90:70)
__device__ __forceinline__ double kick1(double v, double f, double m, double ts2) {
  return __dadd_rn(v, __dmul_rn(__ddiv_rn(__ddiv_rn(f, m), c_mass_coef), ts2));
}
// x = x + v*ts(1) then the shift, rounded as written
__device__ __forceinline__ double drift1(double x, double v, double ts1, double L) {
  return wrap1(__dadd_rn(x, __dmul_rn(v, ts1)), L);
}

template <bool EXACT>
__global__ void k_kick(GroupRef g, int xyz, double ts2, Atoms A, Ctl* ctl) {
  if (ctl->stop) return;
  const int ind = blockIdx.x * blockDim.x + threadIdx.x;
  if (ind >= ctl->group_n[g.g]) return;
  const int i = g.idx[ind];
  const double4_32a f = A.frc[i];
  double4_32a v = A.vel[i];
  if (EXACT) {
    const double m = A.mass[i];
    if (xyz) {
      v.x = kick1(v.x, f.x, m, ts2);
      v.y = kick1(v.y, f.y, m, ts2);
    }
    v.z = kick1(v.z, f.z, m, ts2);
  } else {
    const double kt = A.kc[i] * ts2;
    if (xyz) {
      v.x = kick1_fast(v.x, f.x, kt);
      v.y = kick1_fast(v.y, f.y, kt);
    }
    v.z = kick1_fast(v.z, f.z, kt);
  }
  A.vel[i] = v;
}

__global__ void k_drift(GroupRef g, int xyz, double ts1, int write_posq, Atoms A, Box B, Ctl* ctl) {
  if (ctl->stop) return;
  const int ind = blockIdx.x * blockDim.x + threadIdx.x;
  if (ind >= ctl->group_n[g.g]) return;
  const int i = g.idx[ind];
  const double4_32a v = A.vel[i];
  double4_32a p = A.pos[i];
  if (xyz) {
    p.x = drift1(p.x, v.x, ts1, B.L[0]);
    p.y = drift1(p.y, v.y, ts1, B.L[1]);
  }
  p.z = drift1(p.z, v.z, ts1, B.L[2]);
  A.pos[i] = p;
  if (write_posq) A.posq[i] = make_int4(quantize(p.x, B.qinv[0]), quantize(p.y, B.qinv[1]), quantize(p.z, B.qinv[2]), 0);
  if (out_of_cell(p.x, B.Ltol[0]) || out_of_cell(p.y, B.Ltol[1]) || out_of_cell(p.z, B.Ltol[2])) flag_oob(ctl, i);
}

// Nose-Hoover scaling (optional), half kick and drift of the xyz group in one pass.
// begin: also do k_step_begin's work for an nve step without group changes: every
// thread checks the previous drift's out-of-cell verdict, one thread advances the
// step counter and the previous-step potential energy.
// The atom's force, velocity, position and mass are loaded before the control
// block is read (any index below the group's capacity names a valid atom), so
// those loads overlap instead of forming a chain of dependent round trips.
template <bool EXACT>
__global__ void k_kick_drift(GroupRef g, double ts1, double ts2, int write_posq, int nhc_scale, int begin,
                             int nhc_pre, int early, Atoms A, Box B, Ctl* ctl) {
  asm volatile("griddepcontrol.wait;" ::: "memory");  // see launch_dependent (forces.cuh)
  // early: the next kernel (the fused pair kernel) may start now; it reads its
  // static tables, then waits for this grid to complete
  if (early) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const int ind = blockIdx.x * blockDim.x + threadIdx.x;
  const bool have = ind < g.cap;
  const int i = have ? g.idx[ind] : 0;
  double4_32a f = make_double4_32a(0.0, 0.0, 0.0, 0.0), v = f, p = f;
  double km = 0.0;  // kc (fast kick) or the mass (exact kick)
  if (have) {
    f = A.frc[i];
    v = A.vel[i];
    p = A.pos[i];
    km = EXACT ? A.mass[i] : A.kc[i];
  }
  if (ctl->stop) return;
  if (begin) {
    if (oob_pending(ctl)) {
      // the step counter has not advanced yet: the error belongs to the step begun here
      set_error_at(ctl, ST_OUT_OF_CELL, EK_OOB, ctl->oob_atom + 1, 0, 0, ctl->md_step + 1);
      return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      ctl->md_step = ctl->md_step + 1;
      ctl->pe_prev = ctl->pe_last;
    }
  }
  if (ind >= ctl->group_n[g.g]) return;
  if (nhc_scale) {
    if (nhc_pre) {  // the previous step's second-half scaling, in its own order
      const double sa = ctl->nhc_sa;
      v.x *= sa;
      v.y *= sa;
      v.z *= sa;
    }
    const double s = ctl->nhc[nhc_scale - 1].s;
    v.x *= s;
    v.y *= s;
    v.z *= s;
  }
  if (EXACT) {
    v.x = kick1(v.x, f.x, km, ts2);
    v.y = kick1(v.y, f.y, km, ts2);
    v.z = kick1(v.z, f.z, km, ts2);
  } else {
    const double kt = km * ts2;
    v.x = kick1_fast(v.x, f.x, kt);
    v.y = kick1_fast(v.y, f.y, kt);
    v.z = kick1_fast(v.z, f.z, kt);
  }
  A.vel[i] = v;
  if (EXACT) {
    p.x = drift1(p.x, v.x, ts1, B.L[0]);
    p.y = drift1(p.y, v.y, ts1, B.L[1]);
    p.z = drift1(p.z, v.z, ts1, B.L[2]);
  } else {
    p.x = drift1_fast(p.x, v.x, ts1, B.L[0]);
    p.y = drift1_fast(p.y, v.y, ts1, B.L[1]);
    p.z = drift1_fast(p.z, v.z, ts1, B.L[2]);
  }
  A.pos[i] = p;
  if (write_posq) {
    if (EXACT)
      A.posq[i] = make_int4(quantize(p.x, B.qinv[0]), quantize(p.y, B.qinv[1]), quantize(p.z, B.qinv[2]), 0);
    else
      A.posq[i] = make_int4(quantize_int(p.x, B, 0), quantize_int(p.y, B, 1), quantize_int(p.z, B, 2), 0);
  }
  if (out_of_cell(p.x, B.Ltol[0]) || out_of_cell(p.y, B.Ltol[1]) || out_of_cell(p.z, B.Ltol[2])) flag_oob(ctl, i);
}

// double4 records -> xyz-interleaved arrays, up to three arrays per launch
// (blockIdx.y picks one; null ones are skipped).  One thread per double of the
// interleaved array, so a warp writes 256 contiguous bytes of it: the
// interleaved side may be page-locked host memory reached over NVLink-C2C, where
// whole-line accesses matter; the double4 side is device memory.
struct D4Arrays {
  const double4_32a* d4[3];
  double* xyz[3];
};
__global__ void k_d4_to_xyz(long long n3, D4Arrays a) {
  const int k = blockIdx.y;
  double* xyz = a.xyz[k];
  if (!xyz) return;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  const long long i = t / 3;
  const int c = (int)(t - 3 * i);
  xyz[t] = reinterpret_cast<const double*>(a.d4[k] + i)[c];
}
// pfmd_set_state's conversion in one launch: positions (blockIdx.y 0) and
// velocities (1) from xyz-interleaved doubles, which may be page-locked host
// memory read over the C2C link, into the device records; positions also into
// the fixed-point records.  A block reads its 256 atoms' 768 doubles as three
// coalesced sweeps into shared memory, then each thread writes its atom.
__global__ void __launch_bounds__(256) k_state_in(int n, const double* __restrict__ pos,
                                                  const double* __restrict__ vel, Atoms A, Box B) {
  __shared__ double s[3 * 256];
  const double* src = blockIdx.y == 0 ? pos : vel;
  if (!src) return;
  const long long base = (long long)blockIdx.x * 256;
  const long long m = min(3LL * n - 3 * base, 3LL * 256);
  for (int k = threadIdx.x; k < m; k += 256) s[k] = src[3 * base + k];
  __syncthreads();
  const long long i = base + threadIdx.x;
  if (i >= n) return;
  const double x = s[3 * threadIdx.x], y = s[3 * threadIdx.x + 1], z = s[3 * threadIdx.x + 2];
  if (blockIdx.y == 0) {
    A.pos[i] = make_double4_32a(x, y, z, 0.0);
    A.posq[i] = make_int4(quantize(x, B.qinv[0]), quantize(y, B.qinv[1]), quantize(z, B.qinv[2]), 0);
  } else {
    A.vel[i] = make_double4_32a(x, y, z, 0.0);
  }
}
void launch_state_in(int n, const double* pos, const double* vel, const Atoms& A, const Box& B, cudaStream_t s) {
  if (n <= 0 || (!pos && !vel)) return;
  k_state_in<<<dim3((unsigned)((n + 255) / 256), 2), 256, 0, s>>>(n, pos, vel, A, B);
  ++g_kernel_launches;
}
void launch_d4_to_xyz(int n, const double4_32a* const d4[3], double* const xyz[3], cudaStream_t s) {
  if (n <= 0) return;
  D4Arrays a;
  for (int k = 0; k < 3; ++k) {
    a.d4[k] = d4[k];
    a.xyz[k] = xyz[k];
  }
  const long long n3 = 3LL * n;
  k_d4_to_xyz<<<dim3((unsigned)((n3 + 255) / 256), 3), 256, 0, s>>>(n3, a);
  ++g_kernel_launches;
}


__global__ void k_step_begin_fused(Ctl* ctl) {
  if (ctl->stop) return;
  ctl->md_step = ctl->md_step + 1;
  ctl->pe_prev = ctl->pe_last;
}
void launch_step_begin_fused(Ctl* ctl, cudaStream_t s) {
  k_step_begin_fused<<<1, 1, 0, s>>>(ctl);
  ++g_kernel_launches;
}


// integrate_nose_hoover_chain (md_integrators.f90:200-245) up to the velocity
// scaling: kinetic energy of the chain's group, then nhc_chain_update in the last
// block.  prescale: the velocities first get the chain's pending s (the scaling
// of the chain's previous half, which the force kernel before it left to this
// kernel), so the kinetic energy is that of the scaled velocities, as in the
// reference.  ahead (a step's second half when the next step's first half
// follows with nothing between that changes velocities): the last block also
// runs that first half-update on the kinetic energy after this half's scaling,
// s^2 ke, and leaves both scalings to the next step's kick-drift (Ctl::nhc_sa
// holds this half's s), so neither k_scale nor the next step's k_nhc runs.
__global__ void __launch_bounds__(kRedThreads) k_nhc(int chain, GroupRef g, double ts2, double ts3, double ts4,
                                                     Atoms A, Ctl* ctl, int prescale, int ahead) {
  if (ctl->stop) return;
  const int n = ctl->group_n[g.g];
  const double s0 = ctl->nhc[chain].s;
  double v[1] = {0.0}, out[1];
  for (int ind = blockIdx.x * blockDim.x + threadIdx.x; ind < n; ind += gridDim.x * blockDim.x) {
    const int i = g.idx[ind];
    if (prescale) {
      double4_32a u = A.vel[i];
      u.x *= s0;
      u.y *= s0;
      u.z *= s0;
      A.vel[i] = u;
    }
    v[0] += ke_of(A, i);
  }
  if (!grid_sum<1>(ctl, 0, v, out)) return;
  nhc_chain_update(ctl->nhc[chain], out[0], ts2, ts3, ts4);
  if (ahead) {
    const double sa = ctl->nhc[chain].s;
    ctl->nhc_sa = sa;
    nhc_chain_update(ctl->nhc[chain], out[0] * (sa * sa), ts2, ts3, ts4);
  }
}

// The second half-kick of the xyz-moving group (md_integrators.f90:58-97) fused
// with the Nose-Hoover half-update of the chain over that same group
// (md_integrators.f90:200-245): each thread kicks its atoms and adds their
// kinetic energy after the kick, in k_nhc's grid and order, and the last block
// updates the chain (with ahead, also the next step's first half, as k_nhc).
// One pass over the velocities and one launch instead of two.
template <bool EXACT>
__global__ void __launch_bounds__(kRedThreads) k_kick_nhc(GroupRef g, double kts2, int chain, double ts2, double ts3,
                                                          double ts4, int ahead, Atoms A, Ctl* ctl) {
  if (ctl->stop) return;
  const int n = ctl->group_n[g.g];
  double v[1] = {0.0}, out[1];
  for (int ind = blockIdx.x * blockDim.x + threadIdx.x; ind < n; ind += gridDim.x * blockDim.x) {
    const int i = g.idx[ind];
    const double4_32a f = A.frc[i];
    double4_32a u = A.vel[i];
    if (EXACT) {
      const double m = A.mass[i];
      u.x = kick1(u.x, f.x, m, kts2);
      u.y = kick1(u.y, f.y, m, kts2);
      u.z = kick1(u.z, f.z, m, kts2);
    } else {
      const double kt = A.kc[i] * kts2;
      u.x = kick1_fast(u.x, f.x, kt);
      u.y = kick1_fast(u.y, f.y, kt);
      u.z = kick1_fast(u.z, f.z, kt);
    }
    A.vel[i] = u;
    v[0] += ke_of(A, i);
  }
  if (!grid_sum<1>(ctl, 0, v, out)) return;
  nhc_chain_update(ctl->nhc[chain], out[0], ts2, ts3, ts4);
  if (ahead) {
    const double sa = ctl->nhc[chain].s;
    ctl->nhc_sa = sa;
    nhc_chain_update(ctl->nhc[chain], out[0] * (sa * sa), ts2, ts3, ts4);
  }
}

// scale_velocities (md_general.f90:97-112) by the chain's s
__global__ void k_scale(int chain, GroupRef g, Atoms A, Ctl* ctl) {
  if (ctl->stop) return;
  const int ind = blockIdx.x * blockDim.x + threadIdx.x;
  if (ind >= ctl->group_n[g.g]) return;
  const int i = g.idx[ind];
  const double s = ctl->nhc[chain].s;
  double4_32a v = A.vel[i];
  v.x *= s;
  v.y *= s;
  v.z *= s;
  A.vel[i] = v;
}

// molecular_static_xyz_velocities / _1D_velocities (md_integrators.f90:99-145)
__global__ void k_ms(GroupRef g, int xyz, Atoms A, Ctl* ctl) {
  if (ctl->stop) return;
  const int ind = blockIdx.x * blockDim.x + threadIdx.x;
  if (ind >= ctl->group_n[g.g]) return;
  const int i = g.idx[ind];
  const double4_32a f = A.frc[i];
  double4_32a v = A.vel[i];
  const double fv = f.x * v.x + f.y * v.y + f.z * v.z;
  if (xyz) {
    const double ff = f.x * f.x + f.y * f.y + f.z * f.z;
    if (fv > 0.0 && ff > 1e-12) {
      const double c = fv / ff;
      v.x = c * f.x;
      v.y = c * f.y;
      v.z = c * f.z;
    } else {
      v.x = v.y = v.z = 0.0;
    }
  } else {
    if (!(fv > 0.0)) v.x = v.y = v.z = 0.0;
  }
  A.vel[i] = v;
}

__global__ void k_zero_forces(GroupRef g, Atoms A, Ctl* ctl) {
  if (ctl->stop) return;
  const int ind = blockIdx.x * blockDim.x + threadIdx.x;
  if (ind >= ctl->group_n[g.g]) return;
  A.frc[g.idx[ind]] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
}

// zero_momentum (md_general.f90:236-252): centre-of-mass velocity of the group...
__global__ void __launch_bounds__(kRedThreads) k_momentum(GroupRef g, Atoms A, Ctl* ctl) {
  if (ctl->stop) return;
  const int n = ctl->group_n[g.g];
  double v[4] = {0.0, 0.0, 0.0, 0.0}, out[4];
  for (int ind = blockIdx.x * blockDim.x + threadIdx.x; ind < n; ind += gridDim.x * blockDim.x) {
    const int i = g.idx[ind];
    const double m = A.mass[i];
    const double4_32a u = A.vel[i];
    v[0] += m * u.x;
    v[1] += m * u.y;
    v[2] += m * u.z;
    v[3] += m;
  }
  if (!grid_sum<4>(ctl, 1, v, out)) return;
  ctl->red[12] = out[0] / out[3];
  ctl->red[13] = out[1] / out[3];
  ctl->red[14] = out[2] / out[3];
}
// ...subtracted from every member's velocity
__global__ void k_sub_velocity(GroupRef g, Atoms A, Ctl* ctl) {
  if (ctl->stop) return;
  const int ind = blockIdx.x * blockDim.x + threadIdx.x;
  if (ind >= ctl->group_n[g.g]) return;
  const int i = g.idx[ind];
  double4_32a v = A.vel[i];
  v.x = v.x - ctl->red[12];
  v.y = v.y - ctl->red[13];
  v.z = v.z - ctl->red[14];
  A.vel[i] = v;
}

// md_simulation.f90:191-201: temperature (md_general.f90:301-310), chain energies
// (md_integrators.f90:247-260, nvt only), potential / total / conserved energy.
__global__ void __launch_bounds__(kRedThreads) k_energy_finalize(GroupRef g, int n_inter, int n_nhc, int nvt,
                                                                 Atoms A, Ctl* ctl) {
  if (ctl->stop) return;
  const int n = ctl->group_n[g.g];
  double v[1] = {0.0}, out[1];
  for (int ind = blockIdx.x * blockDim.x + threadIdx.x; ind < n; ind += gridDim.x * blockDim.x)
    v[0] += ke_of(A, g.idx[ind]);
  if (!grid_sum<1>(ctl, 2, v, out)) return;
  const double ke = out[0];
  ctl->ke = ke;
  ctl->temperature = 2 * ke / c_kt_a_degree / (double)(3 * n);
  double enhc = 0.0;
  for (int c = 0; c < n_nhc; ++c) {
    NHCDev& h = ctl->nhc[c];
    if (nvt) {
      const double kt = c_kt_a_degree * h.T;
      double e = h.q[0] / 2 * (h.v[0] * h.v[0]) + 3.0 * h.L * kt * h.x[0];
      for (int i = 1; i < h.M; ++i) e = e + h.q[i] / 2 * (h.v[i] * h.v[i]) + kt * h.x[i];
      h.e = e;
    }
    enhc = enhc + h.e;
  }
  double pe = 0.0;
  for (int k = 0; k < n_inter; ++k) pe = pe + ctl->e_inter[k];
  ctl->pe_last = pe;
  ctl->e_nhc = enhc;
  ctl->total = pe + ke;
  ctl->conserved = ctl->total + enhc;
}

// Output-block sums over the all-atoms group (md_simulation.f90:212-214):
// red[0..2] force sum, red[3..5] sum m*x, red[6..8] sum m*v, red[9] total mass.
__global__ void __launch_bounds__(kRedThreads) k_out_reduce(GroupRef g, Atoms A, Ctl* ctl) {
  const int n = ctl->group_n[g.g];
  double v[10], out[10];
  for (int k = 0; k < 10; ++k) v[k] = 0.0;
  for (int ind = blockIdx.x * blockDim.x + threadIdx.x; ind < n; ind += gridDim.x * blockDim.x) {
    const int i = g.idx[ind];
    const double m = A.mass[i];
    const double4_32a f = A.frc[i], p = A.pos[i], u = A.vel[i];
    v[0] += f.x;
    v[1] += f.y;
    v[2] += f.z;
    v[3] += m * p.x;
    v[4] += m * p.y;
    v[5] += m * p.z;
    v[6] += m * u.x;
    v[7] += m * u.y;
    v[8] += m * u.z;
    v[9] += m;
  }
  if (!grid_sum<10>(ctl, 3, v, out)) return;
  for (int k = 0; k < 10; ++k) ctl->red[k] = out[k];
}
// find_max_velocity (md_general.f90:366-380) over every atom: red[10] = max |v|^2
__global__ void k_max_v2(Atoms A, Ctl* ctl) {
  double m = -1.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.N; i += gridDim.x * blockDim.x) {
    const double4_32a u = A.vel[i];
    m = fmax(m, u.x * u.x + u.y * u.y + u.z * u.z);
  }
  m = warp_max(m);
  // non-negative doubles order like their bit patterns
  if ((threadIdx.x & 31) == 0 && m >= 0.0)
    atomicMax(reinterpret_cast<unsigned long long*>(&ctl->red[10]), (unsigned long long)__double_as_longlong(m));
}

// ---------------- launchers ----------------
static inline int nb(long long n, int bs) { return (int)((n + bs - 1) / bs); }
static inline int red_grid(int cap) {
  int g = nb(cap, kRedThreads);
  return g < 1 ? 1 : (g > kRedBlocks ? kRedBlocks : g);
}

void launch_step_begin(int phase, int n_changes, const ChangeSpec* changes, int nvms, double ms_de, Ctl* ctl,
                       cudaStream_t s) {
  Changes ch;
  ch.n = n_changes < 8 ? n_changes : 8;
  for (int k = 0; k < ch.n; ++k) ch.c[k] = changes[k];
  { k_step_begin<<<1, 1, 0, s>>>(phase, ch, nvms, ms_de, ctl); ++g_kernel_launches; }
}
void launch_check_all(const Atoms& A, const Box& B, Ctl* ctl, cudaStream_t s) {
  if (A.N > 0) { k_check_all<<<nb(A.N, 256), 256, 0, s>>>(A, B, ctl); ++g_kernel_launches; }
}
void launch_invert_z(const Atoms& A, const Box& B, Ctl* ctl, cudaStream_t s) {
  if (A.N > 0) { k_invert_z<<<nb(A.N, 256), 256, 0, s>>>(A, B, ctl); ++g_kernel_launches; }
}
void launch_kick(const GroupRef& g, bool xyz, double ts2, bool exact, const Atoms& A, Ctl* ctl, cudaStream_t s) {
  if (g.cap <= 0) return;
  if (exact)
    k_kick<true><<<nb(g.cap, 256), 256, 0, s>>>(g, xyz ? 1 : 0, ts2, A, ctl);
  else
    k_kick<false><<<nb(g.cap, 256), 256, 0, s>>>(g, xyz ? 1 : 0, ts2, A, ctl);
  ++g_kernel_launches;
}
void launch_drift(const GroupRef& g, bool xyz, double ts1, bool write_posq, const Atoms& A, const Box& B, Ctl* ctl,
                  cudaStream_t s) {
  if (g.cap > 0) { k_drift<<<nb(g.cap, 256), 256, 0, s>>>(g, xyz ? 1 : 0, ts1, write_posq ? 1 : 0, A, B, ctl); ++g_kernel_launches; }
}
void launch_kick_drift(const GroupRef& g, double ts1, double ts2, bool write_posq, int nhc_scale, bool exact,
                       const Atoms& A, const Box& B, Ctl* ctl, cudaStream_t s, bool begin, bool nhc_pre, bool early) {
  if (g.cap <= 0) return;
  if (exact)
    launch_dependent(k_kick_drift<true>, nb(g.cap, 256), 256, s, g, ts1, ts2, write_posq ? 1 : 0, nhc_scale,
                     begin ? 1 : 0, nhc_pre ? 1 : 0, early ? 1 : 0, A, B, ctl);
  else
    launch_dependent(k_kick_drift<false>, nb(g.cap, 256), 256, s, g, ts1, ts2, write_posq ? 1 : 0, nhc_scale,
                     begin ? 1 : 0, nhc_pre ? 1 : 0, early ? 1 : 0, A, B, ctl);
  ++g_kernel_launches;
}
void launch_nhc(int chain, const GroupRef& g, double ts2, double ts3, double ts4, const Atoms& A, Ctl* ctl,
                cudaStream_t s, int prescale, int ahead) {
  {
    k_nhc<<<red_grid(g.cap), kRedThreads, 0, s>>>(chain, g, ts2, ts3, ts4, A, ctl, prescale, ahead);
    ++g_kernel_launches;
  }
}
void launch_kick_nhc(const GroupRef& g, double kts2, bool exact, int chain, double ts2, double ts3, double ts4,
                     bool ahead, const Atoms& A, Ctl* ctl, cudaStream_t s) {
  if (exact)
    k_kick_nhc<true><<<red_grid(g.cap), kRedThreads, 0, s>>>(g, kts2, chain, ts2, ts3, ts4, ahead ? 1 : 0, A, ctl);
  else
    k_kick_nhc<false><<<red_grid(g.cap), kRedThreads, 0, s>>>(g, kts2, chain, ts2, ts3, ts4, ahead ? 1 : 0, A, ctl);
  ++g_kernel_launches;
}
void launch_scale(int chain, const GroupRef& g, const Atoms& A, Ctl* ctl, cudaStream_t s) {
  if (g.cap > 0) { k_scale<<<nb(g.cap, 256), 256, 0, s>>>(chain, g, A, ctl); ++g_kernel_launches; }
}
void launch_ms(const GroupRef& g, bool xyz, const Atoms& A, Ctl* ctl, cudaStream_t s) {
  if (g.cap > 0) { k_ms<<<nb(g.cap, 256), 256, 0, s>>>(g, xyz ? 1 : 0, A, ctl); ++g_kernel_launches; }
}
void launch_zero_forces(const GroupRef& g, const Atoms& A, Ctl* ctl, cudaStream_t s) {
  if (g.cap > 0) { k_zero_forces<<<nb(g.cap, 256), 256, 0, s>>>(g, A, ctl); ++g_kernel_launches; }
}
void launch_zero_momentum(const GroupRef& g, const Atoms& A, Ctl* ctl, cudaStream_t s) {
  { k_momentum<<<red_grid(g.cap), kRedThreads, 0, s>>>(g, A, ctl); ++g_kernel_launches; }
  if (g.cap > 0) { k_sub_velocity<<<nb(g.cap, 256), 256, 0, s>>>(g, A, ctl); ++g_kernel_launches; }
}
__global__ void k_log_row(const Ctl* ctl, double* row) {
  const int t = threadIdx.x;
  if (t < kLogInter) row[6 + t] = ctl->e_inter[t];
  if (t < kLogChains) row[6 + kLogInter + t] = ctl->nhc[t].e;
  if (t == 0) {
    row[0] = ctl->conserved;
    row[1] = ctl->e_nhc;
    row[2] = ctl->total;
    row[3] = ctl->pe_last;
    row[4] = ctl->ke;
    row[5] = ctl->temperature;
  }
}
void launch_log_row(const Ctl* ctl, double* row, cudaStream_t s) {
  k_log_row<<<1, 32, 0, s>>>(ctl, row);
  ++g_kernel_launches;
}
void launch_energy_finalize(const GroupRef& moving, int n_inter, int n_nhc, int nvt, const Atoms& A, Ctl* ctl,
                            cudaStream_t s) {
  { k_energy_finalize<<<red_grid(moving.cap), kRedThreads, 0, s>>>(moving, n_inter, n_nhc, nvt, A, ctl); ++g_kernel_launches; }
}
void launch_out_reduce(const GroupRef& all, const Atoms& A, Ctl* ctl, cudaStream_t s) {
  { k_out_reduce<<<red_grid(all.cap), kRedThreads, 0, s>>>(all, A, ctl); ++g_kernel_launches; }
  cudaMemsetAsync(&ctl->red[10], 0, sizeof(double), s);
  if (A.N > 0) { k_max_v2<<<red_grid(A.N), kRedThreads, 0, s>>>(A, ctl); ++g_kernel_launches; }
}

}  // namespace pfmd
