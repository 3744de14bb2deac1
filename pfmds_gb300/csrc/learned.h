// Learned form: a per-atom neural-network potential standing in for the tb and rjl
// interactions (the classical kernels stay as its fallback and as the check on its
// error).  Each atom's environment within the interaction's own neighbour list is
// described by Behler-Parrinello symmetry functions -- 32 radial
//   G_k = sum_j exp(-eta_k (r_ij - rs_k)^2) fc(r_ij)
// and 16 angular (no r_jk terms)
//   G_a = 2^(1-zeta) sum_{j<k} (1 + lambda cos theta_jik)^zeta exp(-eta (r_ij^2 + r_ik^2)) fc(r_ij) fc(r_ik)
// with fc(r) = (cos(pi r / rc) + 1)/2 -- normalised, and mapped to the atom's
// energy by a 48 -> 64 -> 64 -> 1 network with SiLU activations.  Forces are the
// exact negative gradient of the summed energies: dE/dG by back-propagation through
// the network, then the chain rule through the descriptors, gathered per atom.
#pragma once

#include <string>
#include <vector>

#include "kernels.h"

namespace pfmd {
namespace learned {

constexpr int NR = 32, NA = 16, NG = NR + NA, NH = 64;
constexpr int MAX_ANG = 32;  // angular partners per atom kept in registers

// Besides the baseline (DescPar), a close-contact wall is added to each network's energy: (k/2) (r_core - r)^2 per
// list entry below r_core (each pair sits in both atoms' rows, so a pair's wall
// is k (r_core - r)^2).  r_core is 1.15 A for the tb (C) network and 2.2 A for
// the rjl (Cu) one, in the lower tail of the nearest-neighbour distances that the
// training runs visit; the networks are trained on the classical energies and
// forces minus the wall's, so the wall is part of the model in training and in
// use.  It keeps the dynamics out of the close-contact region that no training
// frame covers, where a network extrapolates freely (without it, an rjl network
// let Cu pairs close to 1.3 A within 900 steps of a 600 K run).
constexpr float kCoreK = 20.f;  // eV/A^2
inline float core_radius(int kind) { return kind == 0 ? 1.15f : 2.2f; }

struct DescPar {
  float rc_rad, rc_ang;
  float rs[NR], eta_r[NR];
  float eta_a[2], zeta[4], lambda[2];  // angular function a = (il*4 + iz)*2 + ie
  float mean[NG], inv_std[NG];
  // pair baseline (rjl networks): the rjl repulsion bA sum_j exp(-bp (r/br0 - 1))
  // fc(r) of each atom, with the reference's cosine switch between bR1 and bR2
  // (RosatoGuillopeLegrand.f90:23-49), is part of the model's energy; the
  // network learns the rest (the embedding term).  bA = 0: no baseline.
  float bA, bp, br0, bR1, bR2;
};
struct Net {
  float W1[NH * NG], b1[NH];
  float W2[NH * NH], b2[NH];
  float w3[NH], b3;
};
struct Model {
  int kind = 0;  // 0: stands in for tb, 1: for rjl
  DescPar d{};
  Net n{};
};

// Descriptor set and a random network for an interaction kind (cut-offs: tb 4.0 A
// radial and angular; rjl 5.0 A radial, 3.0 A angular).
Model default_model(int kind, unsigned seed);
void save_models(const std::string& path, const std::vector<Model>& m);
std::vector<Model> load_models(const std::string& path);

// G (rows x NG, row-major), normalised with d.mean / d.inv_std.
void launch_desc(const ListDev& L, const DescPar* d, const Atoms& A, const Box& B, float* G, Ctl* ctl,
                 cudaStream_t s);
// Per row: energy e[row] and g[row*NG..] = dE/dG (in un-normalised descriptor units).
void launch_mlp(int rows, const float* G, const DescPar* d, const Net* net, float* e, float* g, Ctl* ctl,
                cudaStream_t s);
// The same on the tensor cores (tcgen05, BF16 operands, FP32 accumulation).
void launch_mlp_tc(int rows, const float* G, const DescPar* d, const Net* net, float* e, float* g, Ctl* ctl,
                   cudaStream_t s);
// Forces of the learned energy (store/add and kick per Epi) and, at energy steps,
// the interaction's energy into ctl->e_inter[ekey].  Needs L.row_of.
// leg (nmax x stride, slot-major) and cforce (rows) are scratch of the two passes.
// rcore: the wall's radius (core_radius of the model's kind).
void launch_force(const ListDev& L, const DescPar* d, const float* g, const float* e, float4* leg, float4* cforce,
                  bool energy, const Atoms& A, const Box& B, Ctl* ctl, int eslot, int ekey, cudaStream_t s,
                  const Epi& E, float rcore);

// Training on per-atom energy targets (mean squared error): gradients of one frame
// into grad (sizeof(Net)/4 floats), reduced over rows in a fixed order; *loss_sum
// (device) = sum of squared errors.
struct TrainBuf {
  float* part = nullptr;    // per-block gradient partials (train_blocks(rows) x NET_FLOATS)
  double* lpart = nullptr;  // per-block squared-error partials
  int part_blocks = 0;
  float* grad = nullptr;
  float *m = nullptr, *v = nullptr;  // Adam moments
  double* loss = nullptr;            // [0] sum of squared errors, [1] rows
};
// U (may be null): rows x NG force-matching directions from launch_desc_vjp;
// loss = wE * mean (E - t)^2 + wF * sum |F - F_ref|^2 / (3 N).
void launch_train_grad(int rows, const float* G, const float* U, const double* target_by_row, float wE, float wF,
                       const Net* net, TrainBuf& T, cudaStream_t s);
// Force matching: residuals res = 2 (f_pred - f_ref) / (3 N) per atom, and
// U = inv_std * dL_F/dG per row (needs only the row's own neighbours).
void launch_residual(int n, const double4_32a* fpred, const double4_32a* fref, float4* res, cudaStream_t s);
void launch_desc_vjp(const ListDev& L, const DescPar* d, const Atoms& A, const Box& B, const float4* res, float* U,
                     Ctl* ctl, cudaStream_t s);
// The same gradient on the tensor cores (tcgen05, BF16 operands, FP32 accumulation):
// one persistent CTA per SM, partials per CTA (T.part needs train_tc_grid(rows) rows).
void launch_train_grad_tc(int rows, const float* G, const float* U, const double* target_by_row, float wE, float wF,
                          const Net* net, TrainBuf& T, Ctl* ctl, cudaStream_t s);
int train_tc_grid(int rows);
// Sums `blocks` per-block partials in a fixed order into T.grad and T.loss.
void launch_train_reduce(int blocks, int rows, TrainBuf& T, cudaStream_t s);
void launch_adam(Net* net, TrainBuf& T, int step, float lr, cudaStream_t s);
constexpr int NET_FLOATS = static_cast<int>(sizeof(Net) / sizeof(float));
int train_blocks(int rows);

// Per-row gather of per-atom targets: t[row] = eatom[pidx[row]].
void launch_gather_rows(const ListDev& L, const double* eatom, double* t, cudaStream_t s);
// t[row] -= the row's wall and baseline energy (the network's share of the target).
void launch_core_sub(const ListDev& L, const DescPar* d, const Atoms& A, const Box& B, float rcore, double* t,
                     cudaStream_t s);
// Sum over atoms of |f - f_ref|^2 and |f_ref|^2 (deterministic) into out[0..1].
void launch_force_diff(int n, const double4_32a* f, const double4_32a* fref, double* part, double* out,
                       cudaStream_t s);

}  // namespace learned
}  // namespace pfmd
