/*
 * C ABI of the GB300 monotone-component path (libmpart_gb300.so).
 *
 * Plain pointers, sizes and strides only.  A matrix is (data, rows, cols,
 * row_stride, col_stride) in elements, one column per point, exactly the
 * (ptr, (rows, cols), (rowStride, colStride)) tuples that the reference's
 * Python binding passes to its *Impl methods
 * (bindings/python/package/torch_helpers.py:3-30, MParT/Utilities/ArrayConversions.h:102-115).
 * data may point to device memory or to host memory; host matrices are
 * staged through device buffers inside the call.
 *
 * Every call returns MPGB_OK or a negative error code; mpgb_last_error()
 * gives the message of the last failure on the calling thread.  Calls are
 * ordered on the given CUDA stream (NULL = default stream) and synchronous
 * unless mpgb_set_async(map, 1) was called.
 */
#ifndef MPART_GB300_H
#define MPART_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpgb_map mpgb_map;

enum {
    MPGB_OK = 0,
    MPGB_ERR_INVALID_ARGUMENT = -1, /* std::invalid_argument in the reference */
    MPGB_ERR_RUNTIME = -2,          /* std::runtime_error in the reference */
    MPGB_ERR_CUDA = -3,             /* CUDA runtime failure */
    MPGB_ERR_INTEGRAND = -4         /* g(df) overflowed (MonotoneIntegrand.h:183-190 throws) */
};

enum { MPGB_BASIS_PROBABILIST_HERMITE = 0, MPGB_BASIS_PHYSICIST_HERMITE = 1, MPGB_BASIS_HERMITE_FUNCTIONS = 2 };
enum { MPGB_POS_EXP = 0, MPGB_POS_SOFTPLUS = 1 };
enum { MPGB_QUAD_CLENSHAW_CURTIS = 0, MPGB_QUAD_ADAPTIVE_SIMPSON = 1, MPGB_QUAD_ADAPTIVE_CLENSHAW_CURTIS = 2 };

/* Status bits reported by mpgb_check_status. */
enum {
    MPGB_STATUS_INTEGRAND_INF = 1,
    MPGB_STATUS_INTEGRAND_NAN = 2,
    MPGB_STATUS_QUAD_BUDGET = 4,
    MPGB_STATUS_NO_BRACKET = 8
};

/* MapOptions (MParT/MapOptions.h:58-123); same field meanings and defaults. */
typedef struct mpgb_map_options {
    int basis_type;
    int pos_func_type;
    int quad_type;
    double quad_abs_tol;
    double quad_rel_tol;
    unsigned int quad_max_sub;
    unsigned int quad_min_sub;
    unsigned int quad_pts;
    int cont_deriv;
    int basis_norm;
    double nugget;
    /* Sigmoid expansions (MParT/MapOptions.h:64-73): sigmoid_type 0 = Logistic,
     * edge_type 0 = SoftPlus, edge_shape > 0, sigmoid_sum_type 0 = Linear,
     * 1 = Constant (MParT/Sigmoid.h:45-48). */
    int sigmoid_type;
    int edge_type;
    double edge_shape;
    int sigmoid_sum_type;
} mpgb_map_options;

typedef struct mpgb_matrix {
    double* data;
    int64_t rows;
    int64_t cols;
    int64_t row_stride;
    int64_t col_stride;
} mpgb_matrix;

/* Library version string. */
const char* mpgb_version(void);
/* Message of the last error on this thread. */
const char* mpgb_last_error(void);

/* MapOptions{} defaults (MParT/MapOptions.h:58-123). */
int mpgb_map_options_default(mpgb_map_options* opts);

/* MapFactory::CreateComponent with a compressed FixedMultiIndexSet
 * (src/MapFactory.cpp:22-27; MParT/MultiIndices/FixedMultiIndexSet.h:43-46).
 * nz_starts has num_terms+1 entries. */
int mpgb_create_component(unsigned int dim, unsigned int num_terms, const unsigned int* nz_starts,
                          const unsigned int* nz_dims, const unsigned int* nz_orders, const mpgb_map_options* opts,
                          mpgb_map** out);

/* MapFactory::CreateComponent(FixedMultiIndexSet(dim, order), opts)
 * (src/MultiIndices/FixedMultiIndexSet.cpp:208-233). */
int mpgb_create_component_total_order(unsigned int dim, unsigned int order, const mpgb_map_options* opts,
                                      mpgb_map** out);

/* MapFactory::CreateTriangular (src/MapFactory.cpp:105-124). */
int mpgb_create_triangular(unsigned int input_dim, unsigned int output_dim, unsigned int total_order,
                           const mpgb_map_options* opts, mpgb_map** out);

/* TriangularMap(components, moveCoeffs) (src/TriangularMap.cpp:9-62).  The new
 * map keeps references to the components; their handles stay valid. */
int mpgb_create_triangular_from_components(mpgb_map* const* components, unsigned int n, int move_coeffs,
                                           mpgb_map** out);

/* MapFactory::CreateSigmoidComponent (MParT/MapFactory.h:138-185, src/MapFactory.cpp:256-385):
 * a RectifiedMultivariateExpansion (input_dim >= 2) or UnivariateExpansion
 * (input_dim == 1) with the Sigmoid1d basis built from n_centers centers
 * (CreateSigmoid, src/MapFactory.cpp:181-254) by opts->edge_shape and
 * opts->sigmoid_sum_type.  The first form uses the factory's multi-index set
 * (leading total order off_diag_order, leading cross order cross_order); the
 * second takes the set. */
int mpgb_create_sigmoid_component(unsigned int input_dim, unsigned int off_diag_order, unsigned int cross_order,
                                  const double* centers, unsigned int n_centers, const mpgb_map_options* opts,
                                  mpgb_map** out);
int mpgb_create_sigmoid_component_mset(unsigned int dim, unsigned int num_terms, const unsigned int* nz_starts,
                                       const unsigned int* nz_dims, const unsigned int* nz_orders,
                                       const double* centers, unsigned int n_centers,
                                       const mpgb_map_options* opts, mpgb_map** out);
/* MapFactory::CreateSigmoidTriangular (MParT/MapFactory.h:186-213,
 * src/MapFactory.cpp:389-407): centers is n_centers x output_dim (strides in
 * doubles); column i gives the centers of component i. */
int mpgb_create_sigmoid_triangular(unsigned int input_dim, unsigned int output_dim, unsigned int total_order,
                                   const double* centers, unsigned int n_centers, int64_t row_stride,
                                   int64_t col_stride, const mpgb_map_options* opts, mpgb_map** out);
/* ConditionalMapBase::CoeffBounds (src/ConditionalMapBase.cpp:297-312): host
 * arrays of num_coeffs. */
int mpgb_map_coeff_bounds(const mpgb_map* map, double* lb, double* ub);
/* Kind of a single component: 0 MonotoneComponent, 1 rectified sigmoid
 * expansion, 2 univariate sigmoid expansion; -1 for a TriangularMap. */
int mpgb_map_kind(const mpgb_map* map, int* kind);
/* The Sigmoid1d parameters of a sigmoid component (host arrays of n_centers
 * and n_starts; *n_centers / *n_starts receive the sizes; arrays may be NULL
 * to query them). */
int mpgb_component_sigmoid(const mpgb_map* component, double* centers, double* widths, double* weights,
                           unsigned int* n_centers, unsigned int* starts, unsigned int* n_starts);
/* CreateSigmoid's parameters for a vector of centers (src/MapFactory.cpp:181-254):
 * host arrays of n (starts: room for n); *n_starts receives the start count. */
int mpgb_sigmoid_params(const double* centers, unsigned int n, double edge_shape, int sum_type,
                        double* out_centers, double* widths, double* weights, unsigned int* starts,
                        unsigned int* n_starts);
/* Sigmoid1d::EvaluateAll / EvaluateDerivatives / EvaluateSecondDerivatives
 * (MParT/Sigmoid.h:214-366) on the device: x (device, n_x values, stride
 * x_stride), outputs (device, (max_order+1) x n_x, row stride n_x; d1, d2 may
 * be NULL).  which = 0, 1, 2 selects the derivative order. */
int mpgb_sigmoid1d_evaluate(const double* centers, const double* widths, const double* weights, unsigned int n,
                            const unsigned int* starts, unsigned int n_starts, int which, unsigned int max_order,
                            const double* x, int64_t n_x, int64_t x_stride, double* out, double* d1, double* d2,
                            void* stream);

/* Releases a handle (components held by a triangular map stay alive until it is destroyed). */
int mpgb_map_destroy(mpgb_map* map);

/* inputDim, outputDim, numCoeffs (MParT/ParameterizedFunctionBase.h:184-186). */
int mpgb_map_dims(const mpgb_map* map, unsigned int* input_dim, unsigned int* output_dim, unsigned int* num_coeffs);

/* TriangularMap::NumComponents / GetComponent (MParT/TriangularMap.h:65-66).
 * A component handle must be released with mpgb_map_destroy. */
int mpgb_map_num_components(const mpgb_map* map, unsigned int* n);
/* 1 for a TriangularMap, 0 for a single component. */
int mpgb_map_is_triangular(const mpgb_map* map, int* is_triangular);
int mpgb_map_get_component(mpgb_map* map, unsigned int i, mpgb_map** out);

/* ParameterizedFunctionBase::SetCoeffs, deep copy (src/ParameterizedFunctionBase.cpp:185-207).
 * is_host = 1 when coeffs is a host pointer. */
int mpgb_set_coeffs(mpgb_map* map, const double* coeffs, unsigned int n, int is_host, void* stream);

/* ParameterizedFunctionBase::WrapCoeffs, aliases device memory (src/ParameterizedFunctionBase.cpp:219-228). */
int mpgb_wrap_coeffs(mpgb_map* map, double* device_coeffs, unsigned int n);

/* ParameterizedFunctionBase::CoeffMap (host copy of the coefficients). */
int mpgb_get_coeffs(const mpgb_map* map, double* host_out, unsigned int n);

/* Device pointer of the current coefficients (NULL when unset). */
int mpgb_coeffs_device_ptr(const mpgb_map* map, double** out);

/* 1 = asynchronous calls (no synchronisation or status check inside calls). */
int mpgb_set_async(mpgb_map* map, int async);

/* 1 (default) = points are processed grouped by |x_D| of each component's last
 * input (a stable counting sort on the device) so that warps hold points of
 * similar quadrature cost; 0 = in input order.  Results differ only by
 * summation order. */
int mpgb_set_point_ordering(mpgb_map* map, int on);

/* Synchronise the stream, return and clear the status bits of the last calls. */
int mpgb_check_status(mpgb_map* map, void* stream, int* status);

/* ConditionalMapBase/ParameterizedFunctionBase::EvaluateImpl
 * (MParT/ParameterizedFunctionBase.h:97-98; MonotoneComponent.h:255-299). out is outputDim x N. */
int mpgb_evaluate(mpgb_map* map, mpgb_matrix pts, mpgb_matrix out, void* stream);

/* ConditionalMapBase::LogDeterminantImpl (MParT/ConditionalMapBase.h:96-97). out is 1 x N. */
int mpgb_log_determinant(mpgb_map* map, mpgb_matrix pts, mpgb_matrix out, void* stream);

/* ConditionalMapBase::InverseImpl (MParT/ConditionalMapBase.h:125-127; MonotoneComponent.h:330-443)
 * with the "xtol"/"ytol" options.  x1 has inputDim-outputDim or inputDim rows and N (or 1) columns;
 * info (optional, device int[outputDim*N]) receives the root finder's status per point. */
int mpgb_inverse(mpgb_map* map, mpgb_matrix x1, mpgb_matrix r, mpgb_matrix out, double xtol, double ytol,
                 int* device_info, void* stream);

/* Root solvers of mpgb_inverse_method. */
enum {
    MPGB_INVERSE_BRACKET = 0, /* the reference's "Bracket" method: FindBracket + ITP (RootFinding.h:20-178) */
    MPGB_INVERSE_NEWTON = 1   /* FindBracket, then safeguarded Newton steps with the exact slope dT/dx_D */
};

/* mpgb_inverse with the "Method" option of MonotoneComponent::InverseImpl
 * (MonotoneComponent.h:340-351).  mpgb_inverse uses MPGB_INVERSE_BRACKET, whose
 * iterates are the reference's; MPGB_INVERSE_NEWTON meets the same xtol/ytol
 * stopping rules in about a seventh of the integrand quadratures, at a root
 * that can differ from ITP's by up to xtol + ytol / (dT/dx_D). */
int mpgb_inverse_method(mpgb_map* map, mpgb_matrix x1, mpgb_matrix r, mpgb_matrix out, double xtol, double ytol,
                        int method, int* device_info, void* stream);

/* ParameterizedFunctionBase::CoeffGradImpl (MParT/ParameterizedFunctionBase.h:163-165). out is numCoeffs x N. */
int mpgb_coeff_grad(mpgb_map* map, mpgb_matrix pts, mpgb_matrix sens, mpgb_matrix out, void* stream);

/* ParameterizedFunctionBase::GradientImpl (MParT/ParameterizedFunctionBase.h:133-135). out is inputDim x N. */
int mpgb_gradient(mpgb_map* map, mpgb_matrix pts, mpgb_matrix sens, mpgb_matrix out, void* stream);

/* ConditionalMapBase::LogDeterminantCoeffGradImpl (MParT/ConditionalMapBase.h:151-152). out is numCoeffs x N. */
int mpgb_log_determinant_coeff_grad(mpgb_map* map, mpgb_matrix pts, mpgb_matrix out, void* stream);

/* ConditionalMapBase::LogDeterminantInputGradImpl (MParT/ConditionalMapBase.h:167-168). out is inputDim x N. */
int mpgb_log_determinant_input_grad(mpgb_map* map, mpgb_matrix pts, mpgb_matrix out, void* stream);

/* Fused forward + adjoint: the MpartTorchAutograd forward and backward calls
 * (bindings/python/package/torch_helpers.py:39-114) in one pass.  Any output may
 * have data == NULL.  sens is outputDim x N; logdet_sens is 1 x N (data NULL =
 * logdet_sens_scale for every point).  coeff_grad (numCoeffs doubles, device or
 * host) receives sum_i [sens dT/dc + logdet_sens dlogdet/dc]; input_grad is
 * inputDim x N with the same combination of input gradients. */
int mpgb_fused_fwd_adj(mpgb_map* map, mpgb_matrix pts, mpgb_matrix sens, mpgb_matrix logdet_sens,
                       double logdet_sens_scale, mpgb_matrix out_eval, mpgb_matrix out_logdet, double* coeff_grad,
                       mpgb_matrix input_grad, void* stream);

/* Implicit-function derivative of Inverse (TriangularMap::InverseImpl,
 * src/TriangularMap.cpp:146-184, has no derivative in the reference).  pts is
 * inputDim x N = [x1; x] with x = Inverse(x1, r); w is outputDim x N, the
 * weights of L = sum_{k,i} w(k,i) x(k,i).  coeff_grad (numCoeffs doubles, may
 * be NULL) receives dL/dc = -sum_i lambda_i^T dT/dc(x_i), where
 * (dT/dx)^T lambda = w is solved per point by back-substitution over the
 * components; pts_grad (inputDim x N, data may be NULL) receives
 * [dL/dx1; dL/dr] = [-lambda^T dT/dx1; lambda]. */
int mpgb_inverse_coeff_grad(mpgb_map* map, mpgb_matrix pts, mpgb_matrix w, double* coeff_grad, mpgb_matrix pts_grad,
                            void* stream);

/* FastGaussianReverseKLObjective::ObjectivePlusCoeffGradImpl (src/MapObjective.cpp:221-234)
 * for every component of the map at once.  loss (outputDim doubles) and grad
 * (numCoeffs doubles) may be device or host pointers. */
int mpgb_kl_objective(mpgb_map* map, mpgb_matrix pts, double* loss, double* grad, void* stream);

/* Same results as mpgb_fused_fwd_adj without allocating any memory, for
 * callers that may not allocate while they run (code inside a custom
 * allocator, allocation-free real-time loops, hosts that manage the whole
 * device heap).  No counterpart in the reference.  Scratch comes from a fixed
 * 64 MiB array in device memory that the library holds on every GPU it is
 * loaded on; calls needing more are rejected (MPGB_ERR_INVALID_ARGUMENT).
 * Device pointers of the current device (or managed memory) only;
 * out_logdet only for one-component maps; no input gradient.  All calls
 * share the array, so calls that overlap on the GPU race.  The array's
 * address is looked up once per device when a map is created there, which
 * under CUDA's lazy module loading is when the driver reserves the array; if
 * that look-up failed, the first call on the device makes it (and reserves
 * the array): make that first call during start-up.  Every call reads its
 * status word back and synchronises the stream before returning, so no call
 * can be captured into a CUDA graph. */
int mpgb_fused_fwd_adj_noalloc(mpgb_map* map, mpgb_matrix pts, mpgb_matrix sens, mpgb_matrix logdet_sens,
                               double logdet_sens_scale, mpgb_matrix out_eval, mpgb_matrix out_logdet,
                               double* coeff_grad, void* stream);

/* Training options: limited-memory BFGS per component (NLopt's LD_LBFGS is
 * not available; the stopping fields follow TrainOptions, MParT/TrainMap.h:19-58,
 * with 0 disabling a criterion).  mode 0: one batched launch set per step,
 * replayed from a CUDA graph; 1: batched, direct launches; 2: one fused launch
 * set per component (unbatched); 3: per component, the reference objective's
 * call sequence (FastGaussianReverseKLObjective::CommonEval,
 * src/MapObjective.cpp:185-234: Evaluate, LogDeterminant, CoeffGrad and
 * LogDeterminantCoeffGrad into dense outputs, then reductions). */
/* Optimisation algorithms (TrainOptions::opt_alg, MParT/TrainMap.h:21; NLopt
 * is not used).  MPGB_OPT_SLSQP: the iteration of SLSQP, NLopt's LD_SLSQP and
 * the reference's default, for a problem without constraints (damped-BFGS
 * quasi-Newton with SLSQP's line search); MPGB_OPT_LBFGS: limited-memory BFGS
 * (LD_LBFGS) with `memory` pairs. */
#define MPGB_OPT_SLSQP 0
#define MPGB_OPT_LBFGS 1

typedef struct mpgb_train_options {
    int max_iters;
    int max_evals;
    double ftol_rel;
    double ftol_abs;
    double xtol_rel;
    double xtol_abs;
    double gtol;
    int memory;
    int mode;
    int algorithm;  /* MPGB_OPT_SLSQP (default) or MPGB_OPT_LBFGS */
    int precondition; /* MPGB_OPT_LBFGS: 1 starts every iteration's inverse Hessian from the
                         inverse of the mean squared per-point gradient of each coefficient at
                         the starting coefficients (no counterpart in the reference) */
} mpgb_train_options;

typedef struct mpgb_train_result {
    double total_loss;  /* sum of the component objectives (TrainMap's return value) */
    int iterations;     /* largest number of accepted iterations over the components */
    int evaluations;    /* largest number of objective evaluations over the components */
    int steps;          /* batched objective evaluations performed */
    double ms_per_step; /* device time per step (CUDA events) */
    double total_ms;    /* wall time of the training loop */
    double grad_norm;   /* Euclidean norm of the gradient at the result, over all components */
} mpgb_train_result;

int mpgb_train_options_default(mpgb_train_options* opts);

/* The optimisers of mpgb_train_map on host test problems (no GPU): problem 0 the
 * extended Rosenbrock function from (-1.2, 1, ...) (n even), 1 the quadratic
 * sum_i 10^(4i/(n-1)) (x_i - 1)^2 / 2 from 0.  diag_inverse (n entries or NULL)
 * is the L-BFGS diagonal scaling.  Returns the final point, value and counts. */
int mpgb_optimizer_self_test(int algorithm, int problem, int n, int max_iters, const double* diag_inverse,
                             double* x_out, double* f_out, int* iterations, int* evaluations);

/* TrainMap with a standard-normal KLObjective on a triangular map
 * (src/TrainMap.cpp:144-216): every component minimises its
 * FastGaussianReverseKLObjective.  samples is inputDim x N on the device;
 * loss_per_comp (host, outputDim) receives the final objectives; the map's
 * coefficients are set to the result. */
int mpgb_train_map(mpgb_map* map, mpgb_matrix samples, const mpgb_train_options* opts, double* loss_per_comp,
                   mpgb_train_result* result, void* stream);

/* ------------------------------------------------------------------------
 * Adaptive transport map, TrainMapAdaptive (src/TrainMapAdaptive.cpp:44-271,
 * MParT/TrainMapAdaptive.h:19-47): grows each component's multi-index set one
 * term at a time (the reduced-margin term with the largest KL-gradient
 * magnitude), trains after every addition, keeps the sets with the best test
 * objective, and returns the map of those sets trained from zero.
 * ------------------------------------------------------------------------ */
typedef struct mpgb_atm_options {
    mpgb_map_options map;
    mpgb_train_options train;
    unsigned int max_patience;         /* additions without a better test objective before stopping (10) */
    unsigned int max_size;             /* largest total number of terms (INT_MAX) */
    const unsigned int* max_degrees;   /* inputDim entries (a candidate with any order >= them is skipped) or NULL */
    int verbose;
} mpgb_atm_options;

typedef struct mpgb_atm_result {
    unsigned int size;            /* terms of the returned map */
    unsigned int iterations;      /* terms added during the search */
    double best_test_error;       /* KLObjective::TestError of the best sets during the search */
    double final_train_error;     /* KL objective (with the (M/2) log 2 pi constant) of the returned map */
    double final_test_error;
    double total_ms;
} mpgb_atm_result;

int mpgb_atm_options_default(mpgb_atm_options* opts);

/* The initial sets, one per output (set j has length inputDim - n_sets + j + 1),
 * are given densely: num_terms[j] rows of that length each, all concatenated in
 * multis.  train and test are inputDim x N device matrices (the standard-Gaussian
 * KLObjective of ObjectiveFactory::CreateGaussianKLObjective(train, test)).  The
 * final sets are the returned map's components' multi-index sets
 * (mpgb_component_multi_index); final_num_terms (n_sets, may be NULL) receives their sizes. */
int mpgb_train_map_adaptive(unsigned int n_sets, const unsigned int* num_terms, const unsigned int* multis,
                            mpgb_matrix train, mpgb_matrix test, const mpgb_atm_options* opts, mpgb_map** out,
                            mpgb_atm_result* result, unsigned int* final_num_terms, void* stream);

/* Multi-index sets given densely (n rows of length dim, the active terms in
 * order) are rebuilt as the reference's MultiIndexSet builds them: the terms
 * activated in order, each adding its forward and backward neighbours as
 * inactive entries where they are new (src/MultiIndices/MultiIndexSet.cpp:
 * AddActive, Activate, AddForwardNeighbors, AddBackwardNeighbors), no limiter.
 *
 * Reduced margin: the inactive entries whose existing backward neighbours are
 * all active, in the order the set met them (MultiIndexSet::ReducedMargin,
 * MultiIndexSet.cpp:568-590).  Two-call: out == NULL queries n_out. */
int mpgb_reduced_margin(unsigned int dim, unsigned int n, const unsigned int* multis, unsigned int* n_out,
                        unsigned int* out, unsigned int cap_rows);

/* MultiIndexSet::Expand (MultiIndexSet.cpp:739-766): activates the admissible
 * forward neighbours of the frontier, in the reference's order.  terms_out
 * receives the n_terms_out new terms (rows of length dim, in activation
 * order); idx_out the n_idx_out active indices Expand returns (a term reached
 * from several frontier terms appears once for each, as in the reference).
 * Two-call: terms_out == idx_out == NULL queries the counts; cap bounds both
 * outputs (rows / entries). */
int mpgb_multi_index_expand(unsigned int dim, unsigned int n, const unsigned int* multis, unsigned int* n_terms_out,
                            unsigned int* terms_out, unsigned int* n_idx_out, unsigned int* idx_out,
                            unsigned int cap);

/* Multi-index set of a single component (compressed form); arrays may be NULL to query sizes. */
int mpgb_component_multi_index(const mpgb_map* component, unsigned int* dim, unsigned int* num_terms,
                               unsigned int* nnz, unsigned int* nz_starts, unsigned int* nz_dims,
                               unsigned int* nz_orders);

/* Device time of one KL objective + gradient step of all components in the given mode (see
 * mpgb_train_options.mode) at the map's coefficients, averaged over `steps` steps after three
 * warm-up steps.  loss (outputDim) and grad (numCoeffs), host pointers that may be NULL,
 * receive the objective and gradient of the last step. */
int mpgb_kl_step_time(mpgb_map* map, mpgb_matrix samples, int mode, int steps, double* ms_per_step, double* loss,
                      double* grad, void* stream);

/* FP64 throughput probe: DFMA chains over blocks x threads x iters x 8; writes the
 * kernel time in milliseconds (CUDA events on the stream). */
int mpgb_fp64_probe(int blocks, int threads, int iters, void* stream, float* ms);

/* ------------------------------------------------------------------------
 * Archives (host only; no device work except the coefficient copy of a map).
 * Byte layouts of the reference's cereal binary archives where it has one:
 *   MPGB_ARCHIVE_COEFFS: ParameterizedFunctionBase.Serialize / DeserializeMap
 *     (bindings/python/src/ParameterizedFunctionBase.cpp:51-56,
 *      bindings/python/src/Serialization.cpp:20-31);
 *   options: MapOptions::serialize (MParT/MapOptions.h:126-130);
 *   multi-index sets: FixedMultiIndexSet::save/load
 *     (MParT/MultiIndices/FixedMultiIndexSet.h:115-133).
 *   MPGB_ARCHIVE_MAP for monotone components and triangular maps of them:
 *     the reference's ToBytes / FromBytes / pickle archive,
 *     ParameterizedFunctionBase::Save / Load (MParT/ParameterizedFunctionBase.h:197-215;
 *     bindings/python/src/ParameterizedFunctionBase.cpp:57-79), cereal's
 *     polymorphic encoding of the map with its type names (as
 *     "mpart::TriangularMap<Kokkos::HostSpace>"), the components' expansion,
 *     quadrature, nugget and coefficient view, readable by the reference and
 *     read from it.  The quadrature's integrand dimension in it is the one the
 *     last reference-named operation left (Evaluate, LogDeterminant, ...).
 * MPGB_ARCHIVE_MAP for maps of sigmoid expansions, which the reference does
 * not archive, is this library's own (options, every component's multi-index
 * set and Sigmoid1d arrays, coefficients).  Writers use a two-call
 * convention: *size always receives the archive size, and the bytes are
 * written when buf (cap bytes) is large enough; buf == NULL only queries the
 * size.
 * ------------------------------------------------------------------------ */
enum { MPGB_ARCHIVE_MAP = 0, MPGB_ARCHIVE_COEFFS = 1 };

int mpgb_map_to_bytes(mpgb_map* map, int layout, unsigned char* buf, size_t cap, size_t* size);
/* Rebuilds a component or triangular map from an MPGB_ARCHIVE_MAP archive (either
 * layout) as the reference's Load does: components with the archive's
 * coefficients, triangular maps with its moveCoeffs flag. */
int mpgb_map_from_bytes(const unsigned char* buf, size_t size, mpgb_map** out);
/* Host only (no device): reads a map archive in the reference's layout and
 * writes it again from the description it holds (multi-index sets, options,
 * quadrature state, coefficients and their view label), recomputing every
 * derived field; an archive this library loads comes back unchanged.  Two-call
 * convention as above. */
int mpgb_map_archive_rewrite(const unsigned char* in, size_t in_size, unsigned char* buf, size_t cap, size_t* size);
/* Reads an MPGB_ARCHIVE_COEFFS archive; coeffs (num_coeffs doubles, host) may be NULL to query sizes.
 * The archive of a map without coefficients holds an empty view: coeffs is then not written.
 * MPGB_ARCHIVE_COEFFS writes the map's coefficient view under its label (as the reference's
 * Serialize writes obj.Coeffs()), empty when no coefficients are set. */
int mpgb_coeff_archive_read(const unsigned char* buf, size_t size, unsigned int* input_dim, unsigned int* output_dim,
                            unsigned int* num_coeffs, double* coeffs);
int mpgb_options_to_bytes(const mpgb_map_options* opts, unsigned char* buf, size_t cap, size_t* size);
int mpgb_options_from_bytes(const unsigned char* buf, size_t size, mpgb_map_options* out);
int mpgb_mset_to_bytes(unsigned int dim, unsigned int num_terms, const unsigned int* nz_starts,
                       const unsigned int* nz_dims, const unsigned int* nz_orders, unsigned char* buf, size_t cap,
                       size_t* size);
/* Arrays may be NULL to query dim, num_terms and nnz first. */
int mpgb_mset_from_bytes(const unsigned char* buf, size_t size, unsigned int* dim, unsigned int* num_terms,
                         unsigned int* nnz, unsigned int* nz_starts, unsigned int* nz_dims, unsigned int* nz_orders);

/* ------------------------------------------------------------------------
 * Batch of independent maps (no counterpart in the reference, which runs one
 * map per call): forward, log-determinant and reduced coefficient adjoint of
 * every map in one persistent launch.  Maps may differ in dimension, order and
 * point count but share basis, rectifier and quadrature options; last-
 * coordinate orders up to 8.  Every pointer passed to a batch call is device
 * memory; arrays of matrices and of gradient pointers have one entry per map,
 * and an entry with data == NULL is skipped (sens: no value term).
 * ------------------------------------------------------------------------ */
typedef struct mpgb_batch mpgb_batch;

int mpgb_batch_create(mpgb_map* const* maps, int n, mpgb_batch** out);
int mpgb_batch_destroy(mpgb_batch* batch);

/* coeff_grad[m] (numCoeffs_m doubles) receives
 * sum_i [sens_m dT_m/dc + logdet_sens_scale dlogdet_m/dc] over the points of map m. */
int mpgb_batch_fwd_adj(mpgb_batch* batch, const mpgb_matrix* pts, const mpgb_matrix* sens, double logdet_sens_scale,
                       const mpgb_matrix* out_eval, const mpgb_matrix* out_logdet, double* const* coeff_grad,
                       void* stream);

/* Autotuner: times, on these inputs, block sizes 64 and 128 and 1, 2, 4, 8 or 16
 * tiles of points per work item for every (input dimension, order) bucket of
 * the batch's components, and keeps the fastest; best_ms receives the device
 * time of one launch with the chosen configuration. */
int mpgb_batch_autotune(mpgb_batch* batch, const mpgb_matrix* pts, const mpgb_matrix* sens, double logdet_sens_scale,
                        int reps, double* best_ms, void* stream);

/* The tuning in use: block size, and tiles per item for each bucket (up to max_buckets entries). */
int mpgb_batch_tuning(mpgb_batch* batch, int* tpb, int max_buckets, int* n_buckets, int* dims, int* orders,
                      int* tiles);
int mpgb_batch_set_tuning(mpgb_batch* batch, int tpb, int n_buckets, const int* dims, const int* orders,
                          const int* tiles);

/* Number of kernels this library has launched since it was loaded, over all
 * threads (graph replays count their kernel nodes; launches captured into a
 * graph count nothing).  No counterpart in the reference: it lets a caller
 * confirm how many device launches a call made. */
long long mpgb_launch_count(void);

/* ------------------------------------------------------------------------
 * Reference-structured ("plain") GPU path, the comparator of the fused path:
 * the reference's own structure (MParT/MonotoneComponent.h:255-299, :487-531,
 * :684-741, :824-874) on the device -- per-node term loops over all terms,
 * quadrature of the full numTerms+1 vector with a global per-thread
 * workspace, dense numTerms x N outputs and one launch per operation.
 * One total-order component; device pointers; points are dim x N row-major.
 * ------------------------------------------------------------------------ */
typedef struct mpgb_plain mpgb_plain;
int mpgb_plain_create(unsigned int dim, unsigned int order, const mpgb_map_options* opts, mpgb_plain** out);
int mpgb_plain_destroy(mpgb_plain* plain);
int mpgb_plain_num_terms(const mpgb_plain* plain, unsigned int* n);
/* Evaluate, LogDeterminant, CoeffGrad(sens) and LogDeterminantCoeffGrad as
 * separate launches; coeff_grad receives the column sums of both dense outputs. */
int mpgb_plain_fwd_adj(mpgb_plain* plain, const double* coeffs, const double* pts, long long n_pts,
                       const double* sens, double* out_eval, double* out_logdet, double* coeff_grad, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MPART_GB300_H */
