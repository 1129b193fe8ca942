// engine.cuh -- device data layout and warp-level primitives of the CT-HYB
// pair-move engine (one warp advances one Markov chain).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cthyb {

constexpr int NFMAX = 14;  // flavours (Nd <= 7)
constexpr unsigned FULL = 0xffffffffu;
constexpr double DHUGE = 1.7976931348623157e308;

// status codes stored in the chain header
enum : int {
  ST_OK = 0,
  ST_CAPACITY = 1,     // a proposal would exceed kcap/opcap (state untouched)
  ST_INTERNAL = 2,     // bookkeeping inconsistency (NPairs count, search)
  ST_NUMERIC = 3,      // DetRat too small on an accepted removal (CTQMC.F90:4062)
  ST_UNSUPPORTED = 4,  // move type outside the implemented set
};

struct DModel {
  int nd, nf, ns, nss, nsmax, monomial;
  int mono_lv0;                // every monomial log|value| is zero (density-density models)
  int has_szt;                 // spin flips map superstates to superstates (glob_has_Szt)
  const int* sflip_sst;        // [nss] superstate of the spin-flipped first state (perform_spinflip_check_qn)
  double egs;
  const int* sst_n;            // [nss]
  const int* sst_off;          // [nss]
  const int* connect;          // [nss][nf][2]
  const double* eval;          // [ns]
  const double* evs;           // [ns] eval - egs
  const int* mono_tgt;         // [2nf][ns]
  const double* mono_lv;       // [2nf][ns]
  const unsigned char* mono_neg;
  const long long* blk_off;    // [nss][nf][2]
  const double* blk;
  const long long* dm_off;     // [nss]
  long long dm_size;
};

// Per-chain header (kept in shared memory while a warp works on the chain).
struct Hdr {
  double trace_log, trace_sign, det_log, det_sign, cfgsign;
  double tauwin_min, tauwin_max, taudiff_max;
  double meas_sign;
  int num_windows, window_position, npairs, outer_sst;
  int K, mt_idx, status, nslide;
  int kv, bv;  // dense-block models: ket checkpoints 0..kv and bra checkpoints bv..2^L are valid
  long long nprop, try_add, acc_add, try_rem, acc_rem, qn_add, qn_rem, cnt_meas, logn;
  long long try_glob, acc_glob, qn_glob, try_shift, acc_shift;
  long long try_add4, acc_add4, try_rem4, acc_rem4;
  int k[NFMAX];
  // work counters for the roofline: M bytes, M flops, op-array bytes, tree node updates
  long long w_mbytes, w_mflops, w_opbytes, w_nodes;
  // dense-block trace work: FP64 flops of the block products and bytes of
  // their operands (block, input and output matrices)
  long long w_tflops, w_tbytes;
  // drift control: largest |M_fast - M_rebuilt| and |log|det| fast - rebuilt|
  // seen at the periodic full rebuilds, rebuilds done, determinant-sign
  // disagreements, accepted pair updates since the last rebuild
  double drift_m, drift_det;
  long long n_refresh, refresh_sign_err;
  int acc_since_refresh, pad_refresh;
  // cycles per proposal phase (only with -DCTHYB_PROFILE)
  long long prof[10];
};

struct DGroup {
  int nchains, chain0;
  double beta, hscale, binscale, gscale;  // (nftau-1)/beta, 2^L/beta, ntau/beta
  int nftau;
  const double* hybr;  // [nf][nftau]
  int ntau, ncorr, maxhisto;
  int nleg;            // Legendre coefficients of G measured (NLegMax; 0: none)
  int nscore;          // parameter directions of the score-function dG/dtheta (0: none)
  const double* score_dE;  // [nscore][ns]
  double p_outer, p_global, p_shift;  // PercentageOuterMove, PercentageGlobalMove, PercentageTauShiftMove
  double p_4op;                       // Percentage4OperatorMove
  int offdiag;                        // off-diagonal hybridisation (offdiag = 1)
  const double* hybr_full;            // offdiag: [f1][f2][nftau]
  size_t o_gfull;                     // offdiag: G for every flavour pair [f_a][f_c][ntau]
  int kcap, opcap, L, dense, meas_dm;
  int dmma;            // dense blocks of >= 16 x 16 on the FP64 tensor cores (m8n8k4 MMA)
  int refresh_every;   // accepted pair updates between full rebuilds of M (0: never)
  char* base;          // chain c at base + c*stride
  size_t stride;
  size_t o_hdr, o_mt, o_optau, o_opcode, o_srt_tau, o_srt_slot, o_slot_tau, o_M, o_tree, o_act, o_bstart,
      o_scr, o_gtau, o_histo, o_dm, o_gleg, o_outer, o_dense, o_log, o_glob,  // o_glob: 0 without global/shift moves
      o_glscr,  // per-lane Legendre partial sums (0 when nleg == 0)
      o_chk,    // dense-block models: ket and bra checkpoints at the 2^L + 1 bin edges
      o_score,  // score sums [nscore] and G * score sums [nscore][nf][ntau]
      o_accpair;  // accepted pairs by time difference [nf][ntau] (0: not measured)
  size_t chk_bytes;  // bytes of one checkpoint
  size_t node_bytes;   // bytes of one node slot
  long long logcap;
  const double* empty_w;  // [nss] normalised empty-trace weights
  const double* edges;    // [2^L + 1] time-bin edges beta * j / 2^L
  const long long* ekeys; // [2^L + 1] their order keys (bit patterns)
  int nsym;               // user symmetry moves (with their inverses: 2 * nsym rows)
  const int* symmoves;    // [2 nsym][2 Nd] 1-based target flavours in the reference's order
  int* err_flag;
};

}  // namespace cthyb
