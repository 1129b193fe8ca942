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

}  // namespace cthyb
