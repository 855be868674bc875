/*
 * sps_gnn.h — C ABI of the learned warm start (part of libsps_gb300.so).
 *
 * A bipartite message-passing network over an LP's constraint matrix predicts
 * a PDHG starting point (x0, y0) and a primal weight omega0 for the instances
 * of a parametric LP family (one sparsity pattern, per-instance c / b).  No
 * counterpart in the reference: it always starts PDHG from zero
 * (solver/lp/pdhg.py:175-176); the prediction is consumed by
 * sps_set_warm_start / sps_batch_set_warm_starts, whose cold-start fallback
 * keeps a bad prediction from slowing a solve down.
 *
 * Network (hidden width H, L layers; variable nodes j, constraint nodes i,
 * edges = nonzeros A_ij; a_c = A_ij / deg(i), a_v = A_ij / deg(j)):
 *   hv = relu(Wv fv + bv)                  hc = relu(Wc fc + bc)
 *   per layer l:  hc' = relu(Uc_l hc + Mc_l (sum_j a_c hv) + bc_l)
 *                 hv' = relu(Uv_l hv + Mv_l (sum_i a_v hc') + bv_l)
 *   x0_j = wx . hv_j + bx     y0_i = wy . hc_i + by
 *   log omega0 = wo . [mean_i hc_i, mean_j hv_j] + bo
 * Weights: FP32 master copy (Adam), BF16-rounded copy used by the forward and
 * backward passes, FP32 accumulation everywhere.  Loss per instance:
 *   ax mean_j (x0_j - xt_j)^2 + ay mean_i (y0_i - yt_i)^2 + ao (log omega0 - lt)^2,
 * averaged over the instances of a step.  Feature and target scaling is the
 * caller's (sovereign-solver_gb300/gnn.py).
 *
 * Parameter vector order (FP32): Wv (H x fv), bv (H), Wc (H x fc), bc (H),
 * then per layer Uc, Mc (H x H row-major, out x in), bc_l (H), Uv, Mv, bv_l,
 * then wx (H), bx, wy (H), by, wo (2H), bo.
 */
#ifndef SPS_GNN_H
#define SPS_GNN_H

#include <stdint.h>

#include "sps_pdhg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t n_var, n_con;          /* variable / constraint nodes */
    const int32_t *con_ptr;        /* CSR by constraint: n_con + 1 offsets */
    const int32_t *con_idx;        /*   variable of each edge */
    const float   *con_val;        /*   A_ij of each edge */
    int32_t f_var, f_con;          /* input feature widths (1..8); 1 and 1 with lp_features */
    const int8_t  *con_kind;       /* 1 = '<=' row, 0 = '=' row (NULL = all '='); used by lp_features */
} sps_gnn_graph;

typedef struct {
    int32_t hidden;                /* H: 64 (32 and 64 supported) */
    int32_t layers;                /* L: 1..8, default 3 */
    uint64_t seed;                 /* initialisation */
    float lr, beta1, beta2, eps;   /* Adam */
    float loss_x, loss_y, loss_omega;   /* loss weights */
    int32_t max_batch;             /* instances per call */
    int32_t device;
    int32_t lp_features;           /* 1: the inputs are an LP's scaled costs (var_feat, one per
                                      variable) and right-hand sides (con_feat, one per row); the
                                      device expands them to the network's features
                                      var [c_j, gap_le_j, gap_eq_j, 1], con [b_i, kind_i, cmin_i, 1]
                                      with cmin_i = min of c over row i and gap_le_j / gap_eq_j the
                                      mean of c_j - cmin_i over the '<=' / '=' rows of column j */
    int32_t reserved[5];
} sps_gnn_options;

typedef struct sps_gnn sps_gnn;

int sps_gnn_options_init(sps_gnn_options *opt);
/* Copy the graph to the device and initialise the weights (scaled uniform). */
int sps_gnn_create(const sps_gnn_graph *g, const sps_gnn_options *opt, sps_gnn **out);
/* Forward pass for `batch` instances.  Host arrays, instance-major:
 * var_feat (batch x n_var x f_var), con_feat (batch x n_con x f_con);
 * outputs x0 (batch x n_var), y0 (batch x n_con), log_omega (batch); any
 * output may be NULL. */
int sps_gnn_predict(sps_gnn *g, int32_t batch, const float *var_feat, const float *con_feat,
                    float *x0, float *y0, float *log_omega);
/* Loss and its gradient with respect to the parameter vector (no update).
 * Targets: x_t (batch x n_var), y_t (batch x n_con), log_omega_t (batch). */
int sps_gnn_loss_grad(sps_gnn *g, int32_t batch, const float *var_feat, const float *con_feat,
                      const float *x_t, const float *y_t, const float *log_omega_t,
                      double *loss, float *grad);
/* One Adam step on the loss of `batch` instances; *loss = the loss before the step. */
int sps_gnn_train_step(sps_gnn *g, int32_t batch, const float *var_feat, const float *con_feat,
                       const float *x_t, const float *y_t, const float *log_omega_t, double *loss);
int64_t sps_gnn_num_params(const sps_gnn *g);
/* FP32 master parameters (setting them also refreshes the BF16 copy and resets Adam). */
int sps_gnn_get_params(sps_gnn *g, float *out);
int sps_gnn_set_params(sps_gnn *g, const float *in);
const char *sps_gnn_last_error(const sps_gnn *g);
void sps_gnn_destroy(sps_gnn *g);

/* Warm starts for every instance of a batch predicted on the device: the
 * network's inputs are built from the batch's own data (c / c_scale, b /
 * b_scale), the forward pass runs in chunks of max_batch instances, and the
 * outputs (x0 * x_scale, y0 * y_scale, exp(log_omega)) go straight into the
 * batch's warm-start buffers — nothing crosses the host.  scales = {c_scale,
 * b_scale, x_scale, y_scale}.  The network must use lp_features, live on the
 * batch's device, and every instance must have the network's n and m (same
 * constraint pattern; only the sizes are checked).  The batch's cold-start
 * fallback applies as for sps_batch_set_warm_starts.  Errors:
 * sps_batch_last_error(b). */
int sps_batch_set_warm_starts_gnn(sps_batch *b, sps_gnn *g, const double *scales);

#ifdef __cplusplus
}
#endif
#endif /* SPS_GNN_H */
