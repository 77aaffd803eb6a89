/* Learned AMG parameters: host side of the per-row MLP (gb_mlp.cu).
 *
 * The model maps each row's stencil features to (strength threshold, smoother
 * weight).  With a model set on a BoomerAMG solver, setup takes the mean
 * threshold over the finest level's rows as this setup's strong threshold,
 * and every level's relaxation weight is the mean predicted weight over that
 * level's rows (clamped to [0.1, 0.9] and [0.3, 1.5]).  The training
 * primitives (features, forward, gradient, Adam) work on caller-owned device
 * buffers.  The reference has no learned component. */
#include "gb_internal.h"

#define THETA_MIN 0.1
#define THETA_MAX 0.9
#define W_MIN 0.3
#define W_MAX 1.5

static void *g_bw;          /* BF16 weight copies (device) */
static float *g_part, *g_loss_part;

static int ensure_ws(void)
{
   if (!g_bw)
   {
      g_bw = gb_dmalloc(sizeof(unsigned short) * (size_t) gb_mlp_nbw());
      g_part = (float *) gb_dmalloc(sizeof(float) * (size_t) gb_mlp_grid() * (size_t) gb_mlp_nparam());
      g_loss_part = (float *) gb_dmalloc(sizeof(float) * (size_t) gb_mlp_grid());
   }
   return g_bw ? 0 : 1;
}

static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* mean MLP outputs over the rows of a matrix */
static int predict_means(const float *params, gb_csr *M, double *mean)
{
   cudaStream_t s = gb_stream();
   if (ensure_ws()) { return 1; }
   int n = M->nr;
   void *X = gb_dmalloc(sizeof(unsigned short) * 16 * (size_t) (n > 0 ? n : 1));
   float *out = (float *) gb_dmalloc(sizeof(float) * 2 * (size_t) (n > 0 ? n : 1));
   double *res = (double *) gb_dmalloc(sizeof(double) * 2);
   gb_row_features(n, M->i, M->j, M->v, X, s);
   gb_mlp_pack(params, g_bw, s);
   gb_mlp_forward(n, X, g_bw, params, out, s);
   gb_mean2(n, out, res, s);
   cudaMemcpyAsync(mean, res, sizeof(double) * 2, cudaMemcpyDeviceToHost, s);
   gb_sync();
   gb_dfree(X);
   gb_dfree(out);
   gb_dfree(res);
   return 0;
}

int gb_learn_theta(gb_amg *amg, gb_parcsr *A0, double *theta)
{
   double m[2];
   if (predict_means(amg->mlp_params, &A0->A, m)) { return 1; }
   amg->learned_theta = clampd(m[0], THETA_MIN, THETA_MAX);
   *theta = amg->learned_theta;
   return 0;
}

int gb_learn_weights(gb_amg *amg)
{
   for (int l = 0; l < amg->num_levels; l++)
   {
      double m[2];
      if (predict_means(amg->mlp_params, &amg->lev[l].A->A, m)) { return 1; }
      amg->learned_w[l] = clampd(m[1], W_MIN, W_MAX);
      amg->lev[l].relax_w = amg->learned_w[l];
   }
   return 0;
}

HYPRE_Int HYPRE_GB300_MLPNumParams(HYPRE_Int *n)
{
   if (!n) { gb_error_in_arg(1); return gb_error_flag; }
   *n = gb_mlp_nparam();
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BoomerAMGSetLearnedModel(HYPRE_Solver solver, const HYPRE_Real *params)
{
   gb_amg *a = (gb_amg *) solver;
   if (!a || a->magic != GB_MAGIC_AMG) { gb_error_in_arg(1); return gb_error_flag; }
   if (gb_runtime_init()) { return gb_error_flag; }
   gb_dfree(a->mlp_params);
   a->mlp_params = NULL;
   if (!params) { return gb_error_flag; }
   int np = gb_mlp_nparam();
   float *h = (float *) malloc(sizeof(float) * (size_t) np);
   for (int k = 0; k < np; k++)
   {
      if (params[k] != params[k]) { free(h); gb_error_in_arg(2); return gb_error_flag; }
      h[k] = (float) params[k];
   }
   a->mlp_params = (float *) gb_dmalloc(sizeof(float) * (size_t) np);
   cudaMemcpyAsync(a->mlp_params, h, sizeof(float) * (size_t) np, cudaMemcpyHostToDevice, gb_stream());
   gb_sync();
   free(h);
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BoomerAMGGetLearnedParams(HYPRE_Solver solver, HYPRE_Real *theta, HYPRE_Real *weights,
                                                HYPRE_Int max_levels)
{
   gb_amg *a = (gb_amg *) solver;
   if (!a || a->magic != GB_MAGIC_AMG) { gb_error_in_arg(1); return gb_error_flag; }
   if (!a->mlp_params || !a->setup_done) { gb_error(HYPRE_ERROR_GENERIC, "no learned setup"); return gb_error_flag; }
   if (theta) { *theta = a->learned_theta; }
   if (weights)
   {
      for (int l = 0; l < a->num_levels && l < max_levels; l++) { weights[l] = a->learned_w[l]; }
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_MLPRowFeatures(HYPRE_ParCSRMatrix A, void *features)
{
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(1); return gb_error_flag; }
   if (!features) { gb_error_in_arg(2); return gb_error_flag; }
   gb_row_features(A->A.nr, A->A.i, A->A.j, A->A.v, features, gb_stream());
   gb_cuda_ok(cudaGetLastError(), "MLPRowFeatures");
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_MLPForward(HYPRE_BigInt n, const void *features, const float *params, float *out)
{
   if (n < 0) { gb_error_in_arg(1); return gb_error_flag; }
   if (ensure_ws()) { return gb_error_flag; }
   cudaStream_t s = gb_stream();
   gb_mlp_pack(params, g_bw, s);
   gb_mlp_forward(n, features, g_bw, params, out, s);
   gb_cuda_ok(cudaGetLastError(), "MLPForward");
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_MLPGradient(HYPRE_BigInt n, const void *features, const float *targets, const float *params,
                                  float *grad, float *loss)
{
   if (n < 0) { gb_error_in_arg(1); return gb_error_flag; }
   if (ensure_ws()) { return gb_error_flag; }
   cudaStream_t s = gb_stream();
   gb_mlp_pack(params, g_bw, s);
   if (gb_mlp_grad(n, features, targets, g_bw, params, g_part, g_loss_part, grad, loss, s))
   {
      gb_error(HYPRE_ERROR_GENERIC, "MLPGradient: shared memory opt-in failed");
      return gb_error_flag;
   }
   gb_cuda_ok(cudaGetLastError(), "MLPGradient");
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_MLPAdamStep(float *params, const float *grad, float *m, float *v, HYPRE_Real lr, HYPRE_Int step)
{
   if (step < 1) { gb_error_in_arg(6); return gb_error_flag; }
   gb_mlp_adam(params, grad, m, v, (float) lr, 0.9f, 0.999f, 1e-8f, step, gb_stream());
   gb_cuda_ok(cudaGetLastError(), "MLPAdamStep");
   return gb_error_flag;
}
