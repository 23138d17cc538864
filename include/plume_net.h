/*
 * plume_net.h -- learned pressure warm start for the Poisson solve.
 *
 * No counterpart in the reference: its project step always starts the MIC-PCG
 * solve from p = 0 (FLUID_3D_MIC.cpp:360).  Here a small 3-D U-Net maps the
 * solve's right-hand side (the divergence) to an initial guess; the plain
 * MIC(0)-PCG then runs from that guess to the same stop test, and reruns from
 * p = 0 if it does not converge, so the network changes the iteration count,
 * never the acceptance criterion.
 *
 * Network: 3 levels, 16/32/64 channels, two 3x3x3 convolutions with ReLU per
 * level, 2x2x2 average pooling down, nearest-neighbour upsampling and
 * channel concatenation up, a 1x1x1 output convolution.  BF16 weights and
 * activations, FP32 accumulation (tensor cores), FP32 master weights and
 * Adam.  Input: b / rms(b) on interior cells (channel 0 of 16); output
 * y with x0 = rms(b) * scale * y.  Grid dimensions must be multiples of 4.
 *
 * Training data: (b / rms(b), p / rms(b)) pairs written on the GPU by plain
 * solves of randomised plumes; training runs on the GPU with the network's own
 * forward and backward kernels.
 *
 * Every function returns a plume_status; plume_last_error(NULL) explains
 * failures of calls that take no plume_handle.
 */
#ifndef PLUME_NET_H
#define PLUME_NET_H

#include <stdint.h>

#include "plume.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plume_net plume_net;
typedef struct plume_dataset plume_dataset;

/* A network with seeded He-normal weights and zero biases on `device`. */
int plume_net_create(uint64_t seed, int32_t device, plume_net** out);
void plume_net_destroy(plume_net* net);

/* FP32 master parameters: per convolution W[27][cin][cout] (offset index
   (dz+1)*9 + (dy+1)*3 + (dx+1)) then b[cout], in the order e1a e1b e2a e2b
   b3a b3b d2a d2b d1a d1b; then the output layer's w[16], b. */
int plume_net_num_params(plume_net* net, int64_t* n);
int plume_net_get_params(plume_net* net, float* dst, int64_t n);
int plume_net_set_params(plume_net* net, const float* src, int64_t n);
/* Output scale: x0 = rms(b) * scale * y. */
int plume_net_get_scale(plume_net* net, float* scale);
int plume_net_set_scale(plume_net* net, float scale);
int plume_net_save(plume_net* net, const char* path);
int plume_net_load(plume_net* net, const char* path);

/* Host-buffer forward pass: input and output hold batch * X*Y*Z floats
   (one channel, the reference cell order); input is the normalised
   right-hand side. */
int plume_net_forward(plume_net* net, const int32_t res[3], int32_t batch, const float* input,
                      float* output);

/* Training losses, averaged over the interior cells of every sample, of the
   error e = y - target: */
enum {
  PLUME_LOSS_MSE = 0,    /* e^T e                                              */
  PLUME_LOSS_ENERGY = 1  /* e^T A e + 1e-4 e^T e, A the closed-box 7-point
                            operator: the error norm CG's convergence bound
                            starts from; the small e^T e term pins the constant
                            mode A does not see */
};

/* A loss and its gradient with respect to every parameter
   (plume_net_num_params floats). */
int plume_net_loss_grad(plume_net* net, const int32_t res[3], int32_t batch, int32_t loss_kind,
                        const float* input, const float* target, double* loss, float* grad);

typedef struct plume_dataset_spec {
  int32_t res[3];
  int32_t plumes;   /* randomised plumes (seed + index)                        */
  int32_t steps;    /* steps simulated per plume                               */
  int32_t skip;     /* leading steps of each plume that are not stored         */
  int32_t threads;  /* plumes simulated at once (one handle and stream each)   */
  int32_t device;
  uint64_t seed;
  double tol;       /* rel-L2 stop test of the generating solves               */
  int32_t kind;     /* PLUME_PAIRS_SOLVE, _CORRECTION or _ITERATE              */
} plume_dataset_spec;

/* What a pair (and a network trained on such pairs) maps:
   SOLVE:      b / rms(b) -> p / rms(b)   (the solve's right-hand side to its
               solution; the step uses x0 = scaled network output)
   CORRECTION: r0 / rms(r0) -> (p - p_prev) / rms(r0), r0 = b - A p_prev with
               p_prev the previous step's pressure (the step uses
               x0 = p_prev + scaled network output on r0).
   ITERATE:    r_k / rms(r_k) -> (p - x_k) / rms(r_k), r_k = b - A x_k with x_k
               the iterate after k MIC-PCG iterations of the same solve from
               p = 0, k drawn per pair from 1 .. min(32, half the solve's
               iterations - 1): the residuals a solve meets
               mid-way mapped to their errors, the role of a preconditioner
               stage (PLUME_PRECOND_NET).  A network of this kind used as a
               warm start is applied like a correction network.
   The kind is stored in the network file. */
enum { PLUME_PAIRS_SOLVE = 0, PLUME_PAIRS_CORRECTION = 1, PLUME_PAIRS_ITERATE = 2 };

/* Simulates `plumes` closed-box plumes with the batched-plume randomisation
   (box source centre uniform in the middle third of the floor, buoyancy
   U[0.5, 2], vorticity U[0, 4], +-0.05 seeded noise; FP32 fields, plain
   MIC-PCG) and keeps every solve after `skip` steps as a pair on the GPU. */
int plume_dataset_generate(const plume_dataset_spec* spec, plume_dataset** out);
void plume_dataset_destroy(plume_dataset* ds);
/* Number of pairs, rms of the stored solutions, seconds spent generating. */
int plume_dataset_info(plume_dataset* ds, int32_t* pairs, double* target_rms, double* seconds);
/* One pair to host buffers of X*Y*Z floats (b / rms(b), p / rms(b)). */
int plume_dataset_get_pair(plume_dataset* ds, int32_t index, float* input, float* target);

typedef struct plume_train_spec {
  int32_t epochs;
  int32_t batch;
  int32_t val_pairs; /* the last val_pairs pairs are held out */
  int32_t loss;      /* PLUME_LOSS_MSE or PLUME_LOSS_ENERGY */
  float lr;          /* Adam step size, cosine-decayed to lr_final */
  float lr_final;
  uint64_t seed;     /* shuffle order */
} plume_train_spec;

/* Trains on the dataset's pairs (targets divided by the dataset's solution
   rms, which becomes the network's output scale).  train_loss / val_loss
   (may be NULL) receive one mean loss per epoch. */
int plume_net_train(plume_net* net, plume_dataset* ds, const plume_train_spec* spec, float* train_loss,
                    float* val_loss, double* seconds);

/* Lets `h` use `net` for PLUME_WARM_LEARNED solves (the handle keeps its own
   workspace; the network must outlive the handle and must not be trained
   while attached handles step). */
int plume_attach_net(plume_handle* h, plume_net* net);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_NET_H */
