// model.h -- host-side local problem for the GPU engine.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace cthyb {

struct HostModel {
  int nd = 0, nf = 0, ns = 0, nss = 0, nsmax = 0, monomial = 0;
  int has_szt = 0;                        // QuantumNumbers contains Szt (glob_has_Szt, CTQMC.F90:317-321)
  double egs = 0;
  std::vector<int> sst_n, sst_off;        // per superstate
  std::vector<int> connect;               // [nss][nf][2], flavour f = 2b+s, ca 0=c+ 1=c
  std::vector<double> eval;               // [ns] eigenvalues, superstate-major, ascending
  std::vector<int> fock_of, state_sst;    // [ns]
  std::vector<int> occ_fock;              // [ns] Fock state of occupation-basis vector i (superstate order)
  std::vector<double> evec;               // per superstate n x n column-major eigenvectors, at sst_off^2 offsets
  std::vector<long long> evec_off;        // [nss]
  std::vector<long long> blk_off;         // [nss][nf][2] offset into blk or -1
  std::vector<double> blk;                // dense blocks n_target x n_source, column-major
  std::vector<int> mono_tgt;              // [2nf][ns]
  std::vector<double> mono_lv;            // [2nf][ns]
  std::vector<unsigned char> mono_neg;    // [2nf][ns]
  std::vector<long long> dm_off;          // [nss] offsets of dense rho blocks
  long long dm_size = 0;
};

bool build_model(int nd, const double* umat, const double* muimp, const char* qns, HostModel& m,
                 std::string& err);
void empty_trace_weights(const HostModel& m, double beta, std::vector<double>& w);
// Hamiltonian directions dH/dtheta_p = sum dmuimp_p c+c + 1/2 sum dU_p
// c+c+cc (the operator strings of H) as blocks in the eigenbasis of each
// superstate: out[p * dm_size + dm_off[s] + j * n_s + i] = (V_s^T D_p V_s)(i, j)
// with V_s the eigenvectors.  dumat: np x (2Nd)^4 (each as the U matrix of
// build_model), dmuimp: np x (Nd,2,Nd,2) Fortran order; either may be NULL.
void direction_blocks(const HostModel& m, int np, const double* dumat, const double* dmuimp,
                      std::vector<double>& out);

}  // namespace cthyb
