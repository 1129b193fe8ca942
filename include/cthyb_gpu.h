/* cthyb_gpu.h -- C ABI of the GB300 CT-HYB pair-move engine.
 *
 * Drop-in boundary for the inner Monte Carlo loop of the w2dynamics Fortran
 * module `ctqmc` (src/ctqmc_fortran/CTQMC.F90).  Plain C types only: a
 * Fortran host binds these with iso_c_binding, Python with ctypes.  Every
 * entry returns 0 on success and a negative code on failure; the message is
 * available from cthyb_last_error().  Nothing in the library calls exit,
 * abort or traps: the reference's `stop` conditions (CTQMC.F90:4062
 * "DetRat too small in removal", Trace.F90:1777 "NPairs counting logic
 * error") are reported as CTHYB_ERR_NUMERIC / CTHYB_ERR_INTERNAL.
 *
 * Conventions (as in the reference):
 *   orbital b = 1..Nd, spin s = 1..2, ca = 1 (creator) / 2 (annihilator);
 *   flavour index inside arrays f = 2*(b-1) + (s-1);
 *   Fock bit of (b,s): (b-1) + Nd*(s-1) (Operator.F90:157);
 *   U matrix (2Nd)^4 in Fortran order, flavour 2*(b-1)+s (Trace.F90:449);
 *   muimp (Nd,2,Nd,2) Fortran order, solver sign (cthyb_solver.py:255);
 *   F(tau) (Nd,2,Nftau) Fortran order on tau_j = j*beta/(Nftau-1).
 */
#ifndef CTHYB_GPU_H
#define CTHYB_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CTHYB_OK 0
#define CTHYB_ERR_ARG (-1)
#define CTHYB_ERR_CUDA (-2)
#define CTHYB_ERR_CAPACITY (-3)
#define CTHYB_ERR_NUMERIC (-4)
#define CTHYB_ERR_INTERNAL (-5)
#define CTHYB_ERR_UNSUPPORTED (-6)

typedef struct cthyb_model_s* cthyb_model_t;
typedef struct cthyb_batch_s* cthyb_batch_t;

/* Message of the last failed call on this thread. */
const char* cthyb_last_error(void);

/* Local problem: Fock space, superstates from the QuantumNumbers string,
 * H_loc eigenbasis per superstate, c/c+ blocks in that eigenbasis.
 * Replaces init_States / qns2substates / init_Psi / oneparticle_hamiltonian /
 * u_hamiltonian / diag_Operator / transform_Psis called from init_solver
 * (CTQMC.F90:7894-8000; States.F90:58-186; Operator.F90:115-300,482-546,
 * 637-735,1042-1172).  A string containing "All" partitions the superstates
 * of the other quantum numbers automatically (analyze_hamiltonian,
 * Operator.F90:303-442); an "EPSBLOCK=x" token in the string sets its
 * threshold relative to the largest entry of muimp and U (default 1e-13). */
int cthyb_model_create(int nd, const double* umatrix, const double* muimp,
                       const char* quantum_numbers, cthyb_model_t* out);
int cthyb_model_destroy(cthyb_model_t model);
/* nsst, nstates, nsmax, monomial (1: every c/c+ block has one entry per
 * column -- density-density models), egs */
int cthyb_model_info(cthyb_model_t model, int* nsst, int* nstates, int* nsmax,
                     int* monomial, double* egs);
/* per superstate size/offset; per eigenstate the Fock state with the largest
 * weight and the eigenvalue (StatesSuperstates / EigenstatesEnergies,
 * CTQMC.F90:8040-8060) */
int cthyb_model_states(cthyb_model_t model, int* sst_size, int* sst_offset,
                       int* fock_state, double* evals);
/* Occupation basis and eigenvectors: occ_fock[i] = Fock state (bit
 * (b-1)+Nd*(s-1) set when occupied) of basis vector i in superstate order
 * (States of each superstate, States.F90:58-186; OccbasisMapping,
 * CTQMC.F90:8061); evec (nstates x nstates, column-major, block diagonal)
 * holds the H_loc eigenvectors in that basis, the Evec of
 * Transform_DensityMatrix_EB_to_OCCB (CTQMC.F90:3163-3179).  Either
 * pointer may be NULL. */
int cthyb_model_basis(cthyb_model_t model, int* occ_fock, double* evec);
/* target superstate of operator (b,s,ca) acting on superstate sst, 1-based
 * b, s, ca (the Connect table, States.F90:45), -1 if none */
int cthyb_model_connect(cthyb_model_t model, int sst, int b, int s, int ca);

/* One group of chains sharing beta and F(tau). */
typedef struct {
  double beta;
  int32_t nftau;
  int32_t ntau;          /* G(tau) bins (Ntau) */
  const double* ftau;    /* (Nd,2,Nftau) Fortran order */
  int32_t nchains;
  int32_t seed0;         /* chain c is seeded with seed0 + c unless seeds */
  const int32_t* seeds;  /* optional per-chain seeds (NULL: seed0 + c) */
  double taudiff_max;    /* TaudiffMax parameter; <= 0: one window */
  int32_t ncorr;         /* NCorr: proposals between measurements */
  double p_outer;        /* PercentageOuterMove */
  int32_t kcap;          /* max pairs per flavour (0: automatic) */
  int32_t opcap;         /* max operators in a configuration (0: automatic) */
  int32_t tree_levels;   /* time-bin tree depth, 2^levels leaves (0: automatic, -1: one leaf) */
  int32_t maxhisto;      /* expansion-order histogram bins (MaxHisto) */
  int32_t flags;         /* CTHYB_FLAG_* */
  double p_global;       /* PercentageGlobalMove: spin flip, CA flip, random
                            flavour permutation (StepGlob, CTQMC.F90:4433-4554) */
  double p_shift;        /* PercentageTauShiftMove (StepShiftTau, CTQMC.F90:4557-4835) */
  int32_t nleg;          /* NLegMax: Legendre coefficients of G measured (0: none) */
  int32_t nscore;        /* parameter directions for the score-function dG(tau)/dtheta (0: none;
                            monomial models only, <= 32) */
  const double* score_dE; /* nscore x nstates energy derivatives per eigenstate (row-major) */
  int32_t nsym;          /* NSymMove: user symmetry moves for StepGlob (0: none) */
  const int32_t* symmoves; /* nsym x 2Nd, row i = SymMove(i+1): 1-based target flavour of flavour
                              (b-1) + Nd*(s-1) + 1 (Trace.F90:471-477) */
  double p_4op;          /* Percentage4OperatorMove: share of insertions and removals made as
                            4-operator moves (StepAdd4 / StepRem4, CTQMC.F90:3615-3890, 4153-4431) */
  const double* ftau_full; /* offdiag = 1: F for every flavour pair, (Nd,2,Nd,2,Nftau) Fortran
                              order (NULL: diagonal hybridisation from ftau).  Pair,
                              outer-superstate, global and tau-shift moves (p_4op = 0), GLeg_full
                              for nleg > 0;
                              kcap then bounds the total number of pairs; the inverse matrix over all flavours is in the reference's
                              block order (add_ftau_offset, Trace.F90:3002-3040). */
  int32_t refresh_every; /* drift control (no counterpart in the reference, which rebuilds M
                            exactly only in global moves and set_mc_config): after this many
                            accepted pair updates a chain rebuilds all its inverse matrices from
                            the operator times by Gauss-Jordan elimination (get_InvFullHybr,
                            Trace.F90:2279-2336) and continues with them; 0: every
                            CTHYB_REFRESH_DEFAULT updates, < 0: never.  See cthyb_batch_drift. */
} cthyb_group_desc;

#define CTHYB_REFRESH_DEFAULT 1000

#define CTHYB_FLAG_DENSE 1  /* dense block trace even for monomial models */
#define CTHYB_FLAG_NO_DM 2  /* skip the beta/2 density-matrix measurement */
#define CTHYB_FLAG_DMMA 4   /* dense-block trace: blocks of >= 16 x 16 on the FP64 tensor cores
                               (mma m8n8k4) instead of FP64 fused multiply-adds */
#define CTHYB_FLAG_ACCPAIR 8  /* count accepted pair moves by time difference (AccPair) */

/* Create chains for all groups and initialise them like init_Trace
 * (Trace.F90:340-701): window from TaudiffMax, outer superstate drawn with
 * one uniform number in proportion to the empty trace, NSlide
 * (CTQMC.F90:8069).  Chains are numbered consecutively over groups.
 * Replaces init_solver's init_Trace / init_CTQMC for one process
 * (one chain) or for a batch of independent chains.  The chains' device
 * memory comes from the device's default stream-ordered memory pool, whose
 * release threshold is raised to its maximum so that the next batch of the
 * process reuses it (a process-wide setting of that pool). */
int cthyb_batch_create(cthyb_model_t model, int ngroups, const cthyb_group_desc* groups,
                       cthyb_batch_t* out);
int cthyb_batch_destroy(cthyb_batch_t batch);
int cthyb_batch_nchains(cthyb_batch_t batch);
/* set_taudiffmax (CTQMC.F90:8180 -> init_window, Trace.F90:1608) */
int cthyb_batch_set_taudiffmax(cthyb_batch_t batch, int group, double taudiff_max);
/* ctqmc_warmup(N) for every chain (CTQMC.F90:8188-8263): N pair proposals */
int cthyb_batch_warmup(cthyb_batch_t batch, int64_t nproposals);
/* ctqmc_measure Z-space loop (CTQMC.F90:8355-8566): nmeas x NCorr
 * proposals, measurements of sign, order histogram, density matrix at
 * beta/2 and G(tau) (MeasGtauRem) after each NCorr block.  Accumulates
 * across calls until cthyb_batch_reset_measurements. */
int cthyb_batch_measure(cthyb_batch_t batch, int64_t nmeas);
int cthyb_batch_reset_measurements(cthyb_batch_t batch);
/* Wait for queued work; returns the first chain error if any. */
int cthyb_batch_sync(cthyb_batch_t batch);
/* CUDA stream the batch runs on (cudaStream_t as void*). */
int cthyb_batch_stream(cthyb_batch_t batch, void** stream);
/* Capture the launch sequence of warmup(n) / measure(n) into a CUDA graph
 * once per n and schedule and replay it (1 = on, default off). */
int cthyb_batch_use_graphs(cthyb_batch_t batch, int on);
/* How the sweep kernel schedules chains (no reference counterpart: the
 * Fortran code runs one chain per process).  -1 (default) = automatic
 * (phase-synchronous, two blocks per multiprocessor, at most 16 chains a
 * block); 0 = independent warps, four chains per block; n in 1..32 =
 * phase-synchronous blocks of n chains whose proposals advance phase by
 * phase together.  Per-chain results do not depend on the schedule. */
int cthyb_batch_set_schedule(cthyb_batch_t batch, int warps_per_block);
/* Team sweep (no reference counterpart): warps_per_chain 0 = off (the
 * schedule of cthyb_batch_set_schedule); T in 1..16 = blocks of T warps,
 * each advancing one chain at a time, chains taken from a cost-ordered
 * queue (largest operators x outer-superstate size first) as blocks become
 * free; the T warps evaluate the dense-block trace together.
 * blocks_per_sm bounds the resident blocks per multiprocessor (0: as many
 * as fit), so that blocks take several chains each from the queue.
 * Per-chain results do not depend on it.  cthyb_batch_set_schedule
 * switches it off. */
int cthyb_batch_set_team(cthyb_batch_t batch, int warps_per_chain, int blocks_per_sm);
/* Time `nprop` warmup proposals per chain under each schedule
 * (independent warps; phase-synchronous blocks of 4..32 chains; for
 * dense-block models phase-synchronous blocks of 1..8 chains and team
 * sweeps of 4..16 warps per chain), in two interleaved passes (forward,
 * then reverse order) of nprop/2 each, and keep the fastest; the proposals
 * are real warmup steps of the chains (no reference counterpart), so call
 * it after thermalisation.  *best receives the choice: warps per block of
 * the phase-synchronous schedule (0: independent warps) or
 * 100 + T + 1000 x blocks_per_sm for a team sweep. */
int cthyb_batch_autotune(cthyb_batch_t batch, int64_t nprop, int* best);

/* The remaining Z-space estimators of one chain, normalised as in
 * CTQMC.F90:8740-8760: gleg (Nd,2,nleg) Fortran order (MeasGtauRem's
 * Legendre part, CTQMC.F90:2368-2389), and from MeasOuterHistograms
 * (CTQMC.F90:3285-3341) the outer superstate/state visit histograms
 * (nsst / nstates), their mean signs and their mean trace contributions.
 * Trace contributions are measured for monomial models only (zero
 * otherwise).  Any pointer may be NULL. */
int cthyb_batch_results_extra(cthyb_batch_t batch, int chain, double* gleg, double* outer_sst_histo,
                              double* outer_state_histo, double* sign_sst, double* sign_state,
                              double* contrib_sst, double* contrib_state);

/* Hamiltonian directions theta_p for the trace gradients of dense-block
 * models (no reference counterpart): dH/dtheta_p = sum dmuimp_p c+c +
 * 1/2 sum dU_p c+c+cc, the operator strings of the local Hamiltonian
 * (Operator.F90:482-546, 1042-1108); dumatrix: nparams x (2Nd)^4, each in
 * the layout of cthyb_model_create's umatrix, dmuimp: nparams x
 * (Nd,2,Nd,2) Fortran order (either may be NULL).  Stored in the model as
 * blocks in the eigenbasis of each superstate; nparams <= 32, 0 clears. */
int cthyb_model_set_directions(cthyb_model_t model, int nparams, const double* dumatrix, const double* dmuimp);

/* Per-configuration gradients of log|w| = log|det H| + log|trace| of every
 * chain's current configuration (no reference counterpart: the reference
 * has no derivatives).
 *   grad_delta  (nchains, Nd, 2, Nftau), each chain Fortran order:
 *               d log|det H| / d F(b, s, tau_j), F entering H through the
 *               linear interpolation of get_HybrF (Trace.F90:1014-1033);
 *   grad_params (nchains, nparams): d log|trace| / d theta_p for parameter
 *               directions given, for monomial (density-density) models,
 *               by per-eigenstate energy derivatives dE (nparams x
 *               nstates, row-major, p slowest); for dense-block models
 *               dE = NULL and the directions of cthyb_model_set_directions
 *               (exact derivative of each segment propagator in the
 *               eigenbasis, adjoint sweep from the checkpoints);
 *               nparams <= 32;
 *   log_weights (nchains, 2): log|det H| and the absolute log|trace|
 *               (energies not shifted by the ground-state energy).
 * grad_params/dE may be NULL with nparams = 0. */
int cthyb_batch_gradients(cthyb_batch_t batch, int nparams, const double* dE, double* grad_delta,
                          double* grad_params, double* log_weights);

/* The same with every array in device memory owned by the caller and no
 * host copies (the form a torch.autograd.Function uses): grad_delta_dev
 * (nchains, 2Nd, Nftau) row-major with flavour f = 2(b-1) + (s-1),
 * grad_params_dev (nchains, nparams), log_weights_dev (nchains, 2),
 * dE_dev (nparams, nstates).  Enqueued on `stream` (NULL: the batch's
 * stream) after the batch's queued work; returns without synchronising. */
int cthyb_batch_gradients_device(cthyb_batch_t batch, int nparams, const double* dE_dev, double* grad_delta_dev,
                                 double* grad_params_dev, double* log_weights_dev, void* stream);

/* log|det H| and the absolute log|trace| of every chain's current
 * configuration, (nchains, 2) in device memory, from the weights the chains
 * carry (no kernel walk; the forward value of a torch.autograd.Function
 * whose backward calls cthyb_batch_gradients_device).  Enqueued on `stream`
 * (NULL: the batch's stream) after the batch's queued work. */
int cthyb_batch_log_weights_device(cthyb_batch_t batch, double* lw_dev, void* stream);

/* Score-function estimate of dG(tau)/dtheta_p for the group's parameter
 * directions (nscore > 0): dgtau (nscore, Nd, 2, Ntau), each direction in
 * Fortran order, = <G g_p> - <G><g_p> with g_p = d log|trace| / dtheta_p of
 * the measured configuration, normalised like G(tau); mean_score (nscore)
 * = <g_p>.  Averages over this chain's measurements: for an estimate over
 * several chains combine <G g_p> = dgtau + G <g_p> and G, <g_p> of every
 * chain before subtracting (the covariance of the chains' means belongs to
 * the derivative).  Assumes a sign-free model (configuration sign
 * constant). */
int cthyb_batch_results_score(cthyb_batch_t batch, int chain, double* dgtau, double* mean_score);

/* Global and tau-shift move counters of one chain since the last warmup or
 * measure call: TryGlob, AccGlob, AccQNGlob, TryShift, AccShift
 * (CTQMC.F90:134-136). */
int cthyb_batch_move_counters(cthyb_batch_t batch, int chain, int64_t* counters5);
/* 4-operator move counters since the last warmup/measure call:
 * TryAdd4, AccAdd4, TryRem4, AccRem4 (CTQMC.F90:134-136). */
int cthyb_batch_move_counters4(cthyb_batch_t batch, int chain, int64_t* out4);
/* Off-diagonal groups: G for every flavour pair, (2Nd, 2Nd, Ntau) with index
 * [f_annihilator][f_creator][bin], f = 2(b-1)+(s-1), normalised as
 * Gtau_full (CTQMC.F90:8752-8753; MeasGtauRem_full, CTQMC.F90:2475-2584). */
int cthyb_batch_results_full(cthyb_batch_t batch, int chain, double* gtau_full);
/* Groups with CTHYB_FLAG_ACCPAIR: accepted pair insertions and removals by
 * flavour and time difference, (Nd, 2, Ntau) Fortran order, bin
 * min(Ntau, floor(dtau / beta * Ntau) + 1) (AccPair of the warmup and
 * measurement loops, CTQMC.F90:3579-3582, 4112-4122, 8203-8204; the flavour
 * of the earlier operator of an insertion, of the creator of a removal);
 * counts since the last cthyb_batch_reset_measurements. */
int cthyb_batch_results_accpair(cthyb_batch_t batch, int chain, double* accpair);

/* Off-diagonal groups with nleg > 0: Legendre coefficients of G for every
 * flavour pair, (2Nd, 2Nd, nleg) with index [f_annihilator][f_creator][l],
 * normalised as GLeg_full (CTQMC.F90:8766-8771; measured by
 * MeasGtauRem_full, CTQMC.F90:2533-2555).  The diagonal gleg of
 * cthyb_batch_results_extra stays zero for these groups, as in the
 * reference. */
int cthyb_batch_results_gleg_full(cthyb_batch_t batch, int chain, double* gleg_full);
/* Off-diagonal groups: the inverse matrix over all flavours (rows creators,
 * columns annihilators, block order, column-major k x k); k in *k. */
int cthyb_batch_minv_full(cthyb_batch_t batch, int chain, int* k, double* out);

/* Normalised results of one chain (CTQMC.F90:8676-8760):
 *   gtau (Nd,2,Ntau) Fortran order, mean_sign, densitymatrix in the
 *   eigenbasis (nstates x nstates, column-major), histo (Nd,2,maxhisto)
 *   Fortran order; counters[8] = try_add, acc_add, try_rem, acc_rem,
 *   qn_add, qn_rem, cnt_meas, proposals.  Any output pointer may be NULL. */
int cthyb_batch_results(cthyb_batch_t batch, int chain, double* gtau, double* mean_sign,
                        double* densitymatrix, double* histo, int64_t* counters);
/* Raw (unnormalised) accumulators summed over the chains of one group:
 * gtau_sum[(Nd,2,Ntau)], sign_sum, cnt_meas. */
int cthyb_batch_group_sums(cthyb_batch_t batch, int group, double* gtau_sum,
                           double* sign_sum, int64_t* cnt_meas);
/* Chain state: trace_log, trace_sign, det_log, det_sign, cfgsign, npairs,
 * outer_sst, window_position, num_windows, noper, tauwin_min, tauwin_max,
 * taudiff_max, nslide, status, pairs of flavour 0.. (16 doubles). */
int cthyb_batch_state(cthyb_batch_t batch, int chain, double* out16);
/* Configuration in the get_mc_config layout (CTQMC.F90:9367): returns the
 * operator count in *n; arrays sized by the caller (opcap). */
int cthyb_batch_get_config(cthyb_batch_t batch, int chain, int* n, double* taus,
                           int* orbs, int* spins, int* cas, int* outer_sst);
/* set_mc_config (CTQMC.F90:9378 -> Trace.F90:6872-7001): rebuild lists,
 * full inverse hybridisation matrices by LU, trace and sign. */
int cthyb_batch_set_config(cthyb_batch_t batch, int chain, int n, const double* taus,
                           const int* orbs, const int* spins, const int* cas, int outer_sst);
/* set_mc_config for the chains chain0 .. chain0 + nset - 1 in one call (the
 * warm start of cthyb_solver.py:329-332 with mc_config_inout, for a whole
 * batch): the operators of chain chain0 + i are entries offsets[i] ..
 * offsets[i + 1] - 1 (offsets[0] = 0) of taus/orbs/spins/cas, its outer
 * superstate outer_sst[i].  Every configuration is checked before the
 * first one is written; one upload and one kernel launch per group. */
int cthyb_batch_set_configs(cthyb_batch_t batch, int chain0, int nset, const int* offsets,
                            const double* taus, const int* orbs, const int* spins,
                            const int* cas, const int* outer_sst);
/* get_mc_config for the chains chain0 .. chain0 + nget - 1 (the
 * mc_config_inout read-back, cthyb_solver.py:344-345): fills offsets
 * (nget + 1 entries, as in cthyb_batch_set_configs) and outer_sst (nget,
 * may be NULL); with all four operator arrays NULL only those, else the
 * operators, cap being the arrays' length (CTHYB_ERR_CAPACITY if the
 * total operator count exceeds it). */
int cthyb_batch_get_configs(cthyb_batch_t batch, int chain0, int nget, int* offsets, int cap,
                            double* taus, int* orbs, int* spins, int* cas, int* outer_sst);
/* Inverse hybridisation matrix of one flavour f = 2(b-1)+(s-1) in time
 * order (rows creators, columns annihilators, column-major k x k);
 * returns k in *k. */
int cthyb_batch_minv(cthyb_batch_t batch, int chain, int f, int* k, double* out);
/* Full LU rebuild of every M of every chain (get_InvFullHybr,
 * Trace.F90:2279-2336): max |M_fast - M_LU| over the batch in *maxdev;
 * replace != 0 also installs the rebuilt matrices. */
int cthyb_batch_refresh_minv(cthyb_batch_t batch, int replace, double* maxdev);

/* Per-chain summary of one group (no reference counterpart; what the
 * reference's per-rank outputs hold, for all chains in one copy): out[4*c
 * + 0..3] = operators in the configuration, measurements, sum of the
 * measured signs, proposals since the last warmup/measure call. */
int cthyb_batch_chain_stats(cthyb_batch_t batch, int group, double* out);
/* The raw G(tau) accumulators of every chain of one group in one copy:
 * out[(c * 2Nd + f) * Ntau + bin], f = 2(b-1) + (s-1); chain c's G of
 * cthyb_batch_results is -(raw / cnt) / (-sign_sum / cnt) * Ntau / beta^2
 * with cnt and sign_sum from cthyb_batch_chain_stats (CTQMC.F90:8730). */
int cthyb_batch_group_gtau_raw(cthyb_batch_t batch, int group, double* out);

/* Drift of the fast updates, over all chains since creation or the last
 * reset (no counterpart in the reference): the largest |M_fast - M_rebuilt|
 * element and |log|det H| fast - rebuilt| seen at the periodic rebuilds
 * (refresh_every), the number of rebuilds and of rebuilds whose determinant
 * sign disagreed with the fast-updated one.  reset != 0 clears them after
 * reading.  Any output pointer may be NULL. */
int cthyb_batch_drift(cthyb_batch_t batch, double* max_dev_m, double* max_dev_logdet, int64_t* refreshes,
                      int64_t* sign_errors, int reset);

/* Per-proposal records (layout cthyb_record below) for parity checks:
 * cap records per chain; 0 disables. */
int cthyb_batch_set_log(cthyb_batch_t batch, int64_t cap_per_chain);
int cthyb_batch_get_log(cthyb_batch_t batch, int chain, void* records, int64_t* n);

typedef struct {
  int32_t move, outcome, orb, spin, change_outer, fpos_c, fpos_a, npairs, outer_sst, k_total;
  double tau_c, tau_a, det_log, det_sign, tr_log, tr_sign, prob, rand;
} cthyb_record;

/* Device-side bookkeeping statistics for the roofline, summed over all
 * chains since the last reset (8 int64): bytes of M touched, flops of the
 * determinant ratios and updates, bytes of the operator arrays touched,
 * time-bin tree nodes rebuilt, pair proposals, accepted pair proposals,
 * FP64 flops of the dense-block trace products and bytes of their
 * operands. */
int cthyb_batch_work_counters(cthyb_batch_t batch, int64_t* out8, int reset);

/* FP64 throughput of the running device (no reference counterpart; the
 * denominator of the FP64 rooflines the benchmark reports): GFLOP/s of
 * independent fused multiply-adds on the CUDA cores and of m8n8k4 FP64
 * tensor-core MMAs, best of three timed launches each.  Either pointer may
 * be NULL.  Synchronises the device. */
int cthyb_probe_fp64(double* dfma_gflops, double* dmma_gflops);

/* Allocation-free inverse hybridisation matrix of one flavour -- no
 * counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a solver whose device memory was fixed at start-up, a process whose
 * memory belongs to another allocator, code that must not allocate between
 * capturing and replaying its work): the elimination's two k x k work
 * matrices live in a static device array of the library (1 MiB on every GPU
 * that loads it, kept until exit), so k is limited to 256 and larger k is
 * rejected with CTHYB_ERR_CAPACITY.  All pointers are caller-owned device
 * memory: tau_c[k], tau_a[k] creator/annihilator times, ftau[nftau] F(tau)
 * of the flavour on tau_j = j*beta/(nftau-1); outputs minv[k*k] (column-
 * major, rows creators, columns annihilators, in the order of the inputs)
 * and logdet[2] = log|det H|, sign of H(a,c) = F(tau_a - tau_c).
 * Asynchronous on `stream` (cudaStream_t, NULL for the default stream).
 * The first call on a device resolves the array's device address with that
 * device current and should come before any stream capture; the address is
 * then kept for the life of the process, so it is not valid after a
 * cudaDeviceReset of that device (do not use this entry point after one).
 * Calls share the array: calls whose kernels overlap on the GPU race. */
int cthyb_minv_rebuild_noalloc(int k, const double* tau_c, const double* tau_a, const double* ftau,
                               int nftau, double beta, double* minv, double* logdet, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CTHYB_GPU_H */
