// turb_net.cuh -- the pressure-guess network (k_net.cu) as seen by the solver
// (turb_api.cu): a 4-level 3-D U-Net, channels 16-32-64-128, on the compact
// cell layout of the pressure system.
#pragma once
#include <cuda_runtime.h>

#include "turb_mg.cuh"

struct TurbNet;
struct TurbSnaps;

// records a message for turb_status_string(TURB_ERR_CUDA); returns TURB_ERR_CUDA
int turb_set_error_text(const char *msg);

// kernel launches of one net_guess (norms 4, inputs 1, forward 18, update 1)
constexpr int NET_GUESS_LAUNCHES = 24;

// candidate = base + s * invd * net(r1 / s, (p1 - p2) / |p1 - p2|_rms, b / |b|_rms),
// s = |r1|_rms; all vectors on the compact cell layout of L0
int net_guess(TurbNet *n, cudaStream_t st, const MgDevLevel &L0, const double *invd, const double *r1,
              const double *bw, const double *p1, const double *p2, const double *base, double *out);
// appends the network inputs of this solve to the snapshot store
int net_snapshot(TurbSnaps *sn, cudaStream_t st, const MgDevLevel &L0, const double *invd, const double *r1,
                 const double *bw, const double *p1, const double *p2, const double *base);
// the solve of the pending snapshot ended with pressure p: store its target
// (converged) or drop the snapshot (not converged)
int net_snapshot_finish(TurbSnaps *sn, cudaStream_t st, const MgDevLevel &L0, const double *invd, const double *p,
                        int converged);
int net_dims(const TurbNet *n, int *nx, int *ny, int *nz);
int snaps_dims(const TurbSnaps *s, int *nx, int *ny, int *nz);
int net_train(TurbNet *n, cudaStream_t st, const MgDevLevel &L0, const double *invd, TurbSnaps *sn, int steps,
              float lr, unsigned long long seed, double *mean_loss);
int net_eval(TurbNet *n, cudaStream_t st, const MgDevLevel &L0, const double *invd, TurbSnaps *sn, int first,
             int count, double *mean_res, double *mean_energy);
