// model.cpp -- host-side construction of the local problem.
//
// Builds what w2dynamics' init_solver prepares for the hot loop
// (CTQMC.F90:7894-8000): Fock states, superstates from the QuantumNumbers
// string (States.F90:149-186: grouped in order of first appearance), the
// local Hamiltonian H = sum muimp c+c + 1/2 sum U c+c+cc (Operator.F90:
// 482-546, 1042-1108), its eigenbasis per superstate (DSYEV in
// Operator.F90:637-670; here cyclic Jacobi rotations) and the c/c+ blocks
// rotated into that eigenbasis (transform_Psis, Operator.F90:1130-1172).
//
// Unlike the reference, H is assembled by applying each operator string
// directly to occupation-number bit patterns, and the eigenbasis blocks are
// also stored in "monomial" form (target state, log|value|, sign per source
// state) when every block has one entry per column -- the case of
// density-density interactions, where the GPU trace engine then works with
// state maps instead of dense matrix products.
#include "model.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

namespace cthyb {

namespace {

int popc_below(uint32_t st, int bit) { return __builtin_popcount(st & ((1u << bit) - 1u)); }

// Apply c (ann=true) or c+ of Fock bit `bit` to `st`; returns -1 if zero.
// Sign from the occupied bits below (Operator.F90:157-168).
int apply_op(uint32_t st, int bit, bool ann, double& sign) {
  bool occ = (st >> bit) & 1u;
  if (ann != occ) return -1;
  if (popc_below(st, bit) & 1) sign = -sign;
  return int(st ^ (1u << bit));
}

struct QN {
  bool nt = false, szt = false, qzt = false, azt = false, lzt = false, jzt = false;
};

void qn_values(uint32_t st, int nd, const QN& q, double* v) {
  int n = __builtin_popcount(st);
  double sz = 0, qz = 0, az = 0, lz = 0;
  for (int b = 0; b < nd; ++b) {
    bool up = (st >> b) & 1u, dn = (st >> (b + nd)) & 1u;
    if (up) sz -= 0.5;
    if (dn) sz += 0.5;
    if (up != dn) qz += std::pow(10.0, b);
    if (up) az += std::pow(10.0, b);
    if (dn) az += std::pow(10.0, b + nd);
    double lb = double(b + 1) - double(nd + 1) / 2.0;
    if (up) lz += lb;
    if (dn) lz += lb;
  }
  v[0] = q.nt ? n : 0;
  v[1] = q.szt ? sz : 0;
  v[2] = q.qzt ? qz : 0;
  v[3] = q.azt ? az : 0;
  v[4] = q.lzt ? lz : 0;
  v[5] = q.jzt ? lz + sz : 0;
}

// Cyclic Jacobi eigen-decomposition of a symmetric matrix (column-major),
// eigenvalues ascending, eigenvectors as columns.
void jacobi(int n, std::vector<double>& a, std::vector<double>& w, std::vector<double>& v) {
  v.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
  auto A = [&](int i, int j) -> double& { return a[(size_t)j * n + i]; };
  auto V = [&](int i, int j) -> double& { return v[(size_t)j * n + i]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double x = A(i, j) * A(i, j);
        tot += x;
        if (i != j) off += x;
      }
    if (off <= 1e-30 * (tot + 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = A(p, q);
        if (std::fabs(apq) < 1e-300) continue;
        double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          double akp = A(k, p), akq = A(k, q);
          A(k, p) = c * akp - s * akq;
          A(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = A(p, k), aqk = A(q, k);
          A(p, k) = c * apk - s * aqk;
          A(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V(k, p), vkq = V(k, q);
          V(k, p) = c * vkp - s * vkq;
          V(k, q) = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return A(x, x) < A(y, y); });
  std::vector<double> vs((size_t)n * n);
  w.resize(n);
  for (int k = 0; k < n; ++k) {
    w[k] = A(idx[k], idx[k]);
    for (int i = 0; i < n; ++i) vs[(size_t)k * n + i] = v[(size_t)idx[k] * n + i];
  }
  v.swap(vs);
}

// H = sum muimp c+c + 1/2 sum U c+c+cc in the occupation basis, one block
// per superstate of the partition `sst_of` (states of each superstate in
// `members` order), by applying each operator string to bit patterns.
// As the reference assembles H from its superstate connections
// (Operator.F90:482-546, 1042-1108), every operator of a string must move
// the state to another superstate (a superstate's Connect entry is never
// the superstate itself, Operator.F90:146), and entries that leave a
// superstate are dropped (Operator.F90:1077-1084).  Under quantum numbers
// that include Nt every operator changes the superstate, so only the
// second rule ever applies there.
void assemble_h(int nd, const double* umat, const double* muimp, const std::vector<int>& sst_of,
                const std::vector<std::vector<uint32_t>>& members, std::vector<std::vector<double>>& H) {
  const int nf = 2 * nd, ns = 1 << (2 * nd), nss = (int)members.size();
  std::vector<int> pos_in_sst(ns);
  for (int s = 0; s < nss; ++s)
    for (size_t i = 0; i < members[s].size(); ++i) pos_in_sst[members[s][i]] = (int)i;
  H.assign(nss, {});
  for (int s = 0; s < nss; ++s) H[s].assign(members[s].size() * members[s].size(), 0.0);
  auto add_entry = [&](uint32_t from, int to, double v) {
    const int sf = sst_of[from];
    if (sst_of[to] != sf) return;
    const size_t n = members[sf].size();
    H[sf][(size_t)pos_in_sst[from] * n + pos_in_sst[to]] += v;
  };
  auto bit_of = [&](int fl) { return (fl / 2) + nd * (fl % 2); };
  for (int f1 = 0; f1 < nf; ++f1)
    for (int f2 = 0; f2 < nf; ++f2) {
      // muimp(b1,s1,b2,s2) Fortran order
      const int b1 = f1 / 2, s1 = f1 % 2, b2 = f2 / 2, s2 = f2 % 2;
      const double v = muimp[b1 + nd * (s1 + 2 * (b2 + nd * s2))];
      if (v == 0.0) continue;
      for (int st = 0; st < ns; ++st) {
        double sg = 1.0;
        const int a = apply_op(st, bit_of(f2), true, sg);
        if (a < 0 || sst_of[a] == sst_of[st]) continue;
        const int c = apply_op(a, bit_of(f1), false, sg);
        if (c < 0 || sst_of[c] == sst_of[a]) continue;
        add_entry(st, c, v * sg);
      }
    }
  for (int i = 0; i < nf; ++i)
    for (int j = 0; j < nf; ++j)
      for (int k = 0; k < nf; ++k)
        for (int l = 0; l < nf; ++l) {
          const double u = umat[i + nf * (j + nf * (k + nf * l))];
          if (u == 0.0) continue;
          // 1/2 U_ijkl c+_i c+_j c_l c_k
          for (int st = 0; st < ns; ++st) {
            double sg = 1.0;
            int x = apply_op(st, bit_of(k), true, sg);
            if (x < 0 || sst_of[x] == sst_of[st]) continue;
            int y = apply_op(x, bit_of(l), true, sg);
            if (y < 0 || sst_of[y] == sst_of[x]) continue;
            x = apply_op(y, bit_of(j), false, sg);
            if (x < 0 || sst_of[x] == sst_of[y]) continue;
            y = apply_op(x, bit_of(i), false, sg);
            if (y < 0 || sst_of[y] == sst_of[x]) continue;
            add_entry(st, y, 0.5 * u * sg);
          }
        }
  // force_hermitian
  for (int s = 0; s < nss; ++s) {
    const size_t n = members[s].size();
    std::vector<double>& h = H[s];
    for (size_t i = 0; i < n; ++i)
      for (size_t j = i + 1; j < n; ++j) {
        const double a = 0.5 * (h[j * n + i] + h[i * n + j]);
        h[j * n + i] = h[i * n + j] = a;
      }
  }
}

// QuantumNumbers containing "All": automatic block partitioning
// (analyze_hamiltonian, Operator.F90:303-442, called by init_solver,
// CTQMC.F90:7971-7990).  Each superstate of the given partition splits
// into the connected components of its Hamiltonian (entries of magnitude
// above `threshold`), numbered in order of discovery from the lowest
// unassigned state; then blocks are joined until every creator and
// annihilator maps each block into a single block (the targets of two
// states of one block are merged).  Joining keeps the lower number and
// closes the gaps, so the final blocks are numbered by the smallest
// component number they contain; here the joins run on a union-find forest
// to the same fixed point.  States of a block in ascending order.
void partition_all(int nd, const double* umat, const double* muimp, double threshold, std::vector<int>& sst_of,
                   std::vector<std::vector<uint32_t>>& members) {
  const int ns = 1 << (2 * nd);
  std::vector<std::vector<double>> H;
  assemble_h(nd, umat, muimp, sst_of, members, H);
  std::vector<int> comp(ns, -1);
  int ncomp = 0;
  for (size_t s = 0; s < members.size(); ++s) {
    const int n = (int)members[s].size();
    std::vector<int> local(n, -1);
    for (int start = 0; start < n; ++start) {
      if (local[start] >= 0) continue;
      const int id = ncomp++;
      std::vector<int> net = {start};
      local[start] = id;
      for (size_t q = 0; q < net.size(); ++q) {
        const int node = net[q];
        for (int e = 0; e < n; ++e) {
          const double h = H[s][(size_t)node * n + e];
          if (h != 0.0 && std::fabs(h) > threshold && local[e] < 0) {
            local[e] = id;
            net.push_back(e);
          }
        }
      }
    }
    for (int i = 0; i < n; ++i) comp[members[s][i]] = local[i];
  }
  std::vector<int> parent(ncomp);
  for (int i = 0; i < ncomp; ++i) parent[i] = i;
  auto find = [&](int x) {
    while (parent[x] != x) x = parent[x] = parent[parent[x]];
    return x;
  };
  bool change = true;
  while (change) {
    change = false;
    for (int bit = 0; bit < 2 * nd; ++bit)
      for (int ann = 0; ann < 2; ++ann) {
        // first target block seen for each source block
        std::vector<int> tgt(ncomp, -1);
        for (int st = 0; st < ns; ++st) {
          double sg = 1.0;
          const int r = apply_op(st, bit, ann == 1, sg);
          if (r < 0) continue;
          const int a = find(comp[st]), t = find(comp[r]);
          if (tgt[a] < 0) {
            tgt[a] = t;
          } else if (find(tgt[a]) != t) {
            const int u = find(tgt[a]);
            parent[std::max(u, t)] = std::min(u, t);
            change = true;
          }
        }
      }
  }
  // final numbering: blocks ordered by their smallest component number
  std::vector<int> rank(ncomp, -1);
  int nb = 0;
  for (int c = 0; c < ncomp; ++c) {
    const int r = find(c);
    if (rank[r] < 0) rank[r] = nb++;
  }
  members.assign(nb, {});
  for (int st = 0; st < ns; ++st) {
    sst_of[st] = rank[find(comp[st])];
    members[sst_of[st]].push_back((uint32_t)st);
  }
}

}  // namespace

bool build_model(int nd, const double* umat, const double* muimp, const char* qns, HostModel& m,
                 std::string& err) {
  if (nd < 1 || nd > 7) {
    err = "Nd must be in 1..7";
    return false;
  }
  m.nd = nd;
  m.nf = 2 * nd;
  m.ns = 1 << (2 * nd);
  std::string q(qns ? qns : "");
  const bool all = q.find("All") != std::string::npos;
  double epsblock = 1e-13;  // EPSBLOCK default (configspec)
  {
    const size_t e = q.find("EPSBLOCK=");
    if (e != std::string::npos) epsblock = std::strtod(q.c_str() + e + 9, nullptr);
  }
  QN qf;
  qf.nt = q.find("Nt") != std::string::npos;
  qf.szt = q.find("Szt") != std::string::npos;
  m.has_szt = qf.szt ? 1 : 0;
  qf.qzt = q.find("Qzt") != std::string::npos;
  qf.azt = q.find("Azt") != std::string::npos;
  qf.lzt = q.find("Lzt") != std::string::npos;
  qf.jzt = q.find("Jzt") != std::string::npos;
  const int ns = m.ns, nf = m.nf;
  // superstates in order of first appearance of their quantum numbers
  std::vector<int> sst_of(ns, -1);
  std::vector<std::vector<uint32_t>> members;
  std::vector<double> vals((size_t)ns * 6);
  for (int st = 0; st < ns; ++st) qn_values(st, nd, qf, &vals[(size_t)st * 6]);
  for (int st = 0; st < ns; ++st) {
    if (sst_of[st] >= 0) continue;
    int id = (int)members.size();
    members.push_back({});
    for (int s2 = st; s2 < ns; ++s2) {
      if (sst_of[s2] >= 0) continue;
      bool same = true;
      for (int k = 0; k < 6; ++k)
        if (std::fabs(vals[(size_t)st * 6 + k] - vals[(size_t)s2 * 6 + k]) >= 1e-12) same = false;
      if (same) {
        sst_of[s2] = id;
        members[id].push_back((uint32_t)s2);
      }
    }
  }
  if (all) {
    // threshold relative to the largest entry of muimp and U (CTQMC.F90:7972-7975)
    double mx = 0.0;
    for (int i = 0; i < nf * nf; ++i) mx = std::max(mx, std::fabs(muimp[i]));
    for (int i = 0; i < nf * nf * nf * nf; ++i) mx = std::max(mx, std::fabs(umat[i]));
    partition_all(nd, umat, muimp, epsblock * mx, sst_of, members);
  }
  const int nss = (int)members.size();
  m.nss = nss;
  m.sst_n.resize(nss);
  m.sst_off.resize(nss);
  int off = 0;
  m.nsmax = 0;
  std::vector<int> pos_in_sst(ns);
  for (int s = 0; s < nss; ++s) {
    m.sst_n[s] = (int)members[s].size();
    m.sst_off[s] = off;
    for (int i = 0; i < m.sst_n[s]; ++i) pos_in_sst[members[s][i]] = i;
    off += m.sst_n[s];
    m.nsmax = std::max(m.nsmax, m.sst_n[s]);
  }
  // connection table: op (f, ca) maps superstate s to a unique target
  m.connect.assign((size_t)nss * nf * 2, -1);
  for (int s = 0; s < nss; ++s)
    for (int b = 0; b < nd; ++b)
      for (int sp = 0; sp < 2; ++sp)
        for (int ca = 0; ca < 2; ++ca) {
          int f = 2 * b + sp, bit = b + nd * sp, tgt = -1;
          for (uint32_t st : members[s]) {
            double sg = 1.0;
            int r = apply_op(st, bit, ca == 1, sg);
            if (r < 0) continue;
            int t = sst_of[r];
            if (tgt >= 0 && t != tgt) {
              err = "quantum numbers do not block the creation/annihilation operators";
              return false;
            }
            tgt = t;
          }
          // a superstate never connects to itself (Operator.F90:146)
          m.connect[((size_t)s * nf + f) * 2 + ca] = tgt == s ? -1 : tgt;
        }
  // Hamiltonian blocks by acting on bit patterns (symmetrised)
  std::vector<std::vector<double>> H;
  assemble_h(nd, umat, muimp, sst_of, members, H);
  auto bit_of = [&](int fl) { return (fl / 2) + nd * (fl % 2); };
  // diagonalise
  m.eval.assign(ns, 0.0);
  std::vector<std::vector<double>> V(nss);
  m.egs = 1e300;
  for (int s = 0; s < nss; ++s) {
    int n = m.sst_n[s];
    std::vector<double>& h = H[s];
    std::vector<double> w;
    jacobi(n, h, w, V[s]);
    for (int i = 0; i < n; ++i) m.eval[m.sst_off[s] + i] = w[i];
    m.egs = std::min(m.egs, w[0]);
  }
  // occupation basis and eigenvectors (Evec of Transform_DensityMatrix_EB_to_OCCB)
  m.occ_fock.resize(ns);
  m.evec_off.assign(nss, 0);
  m.evec.clear();
  for (int s = 0; s < nss; ++s) {
    for (int i = 0; i < m.sst_n[s]; ++i) m.occ_fock[m.sst_off[s] + i] = (int)members[s][i];
    m.evec_off[s] = (long long)m.evec.size();
    m.evec.insert(m.evec.end(), V[s].begin(), V[s].end());
  }
  // dominant Fock state per eigenstate
  m.fock_of.resize(ns);
  m.state_sst.resize(ns);
  for (int s = 0; s < nss; ++s) {
    int n = m.sst_n[s];
    for (int k = 0; k < n; ++k) {
      int best = 0;
      for (int i = 1; i < n; ++i)
        if (std::fabs(V[s][(size_t)k * n + i]) > std::fabs(V[s][(size_t)k * n + best])) best = i;
      m.fock_of[m.sst_off[s] + k] = (int)members[s][best];
      m.state_sst[m.sst_off[s] + k] = s;
    }
  }
  // c/c+ blocks in the eigenbasis: B = V_t^T C V_s
  m.blk_off.assign((size_t)nss * nf * 2, -1);
  m.blk.clear();
  m.monomial = 1;
  for (int s = 0; s < nss; ++s)
    for (int f = 0; f < nf; ++f)
      for (int ca = 0; ca < 2; ++ca) {
        int t = m.connect[((size_t)s * nf + f) * 2 + ca];
        if (t < 0) continue;
        int n1 = m.sst_n[s], n2 = m.sst_n[t];
        std::vector<double> C((size_t)n2 * n1, 0.0);
        for (int i = 0; i < n1; ++i) {
          double sg = 1.0;
          int r = apply_op(members[s][i], bit_of(f), ca == 1, sg);
          if (r < 0) continue;
          C[(size_t)i * n2 + pos_in_sst[r]] = sg;
        }
        std::vector<double> CV((size_t)n2 * n1, 0.0), B((size_t)n2 * n1, 0.0);
        for (int j = 0; j < n1; ++j)
          for (int k = 0; k < n1; ++k) {
            double v = V[s][(size_t)j * n1 + k];
            if (v == 0.0) continue;
            for (int i = 0; i < n2; ++i) CV[(size_t)j * n2 + i] += C[(size_t)k * n2 + i] * v;
          }
        for (int j = 0; j < n1; ++j)
          for (int i = 0; i < n2; ++i) {
            double acc = 0;
            for (int k = 0; k < n2; ++k) acc += V[t][(size_t)i * n2 + k] * CV[(size_t)j * n2 + k];
            B[(size_t)j * n2 + i] = acc;
          }
        // flush rounding dust so that exact monomial structure is detected
        double mx = 0;
        for (double x : B) mx = std::max(mx, std::fabs(x));
        for (double& x : B)
          if (std::fabs(x) < 1e-14 * mx) x = 0.0;
        for (int j = 0; j < n1; ++j) {
          int nz = 0;
          for (int i = 0; i < n2; ++i) nz += B[(size_t)j * n2 + i] != 0.0;
          if (nz > 1) m.monomial = 0;
        }
        for (int i = 0; i < n2; ++i) {
          int nz = 0;
          for (int j = 0; j < n1; ++j) nz += B[(size_t)j * n2 + i] != 0.0;
          if (nz > 1) m.monomial = 0;
        }
        m.blk_off[((size_t)s * nf + f) * 2 + ca] = (long long)m.blk.size();
        m.blk.insert(m.blk.end(), B.begin(), B.end());
      }
  // monomial tables: code = 2f + ca, per global eigenstate
  m.mono_tgt.assign((size_t)2 * nf * ns, -1);
  m.mono_lv.assign((size_t)2 * nf * ns, 0.0);
  m.mono_neg.assign((size_t)2 * nf * ns, 0);
  if (m.monomial) {
    for (int s = 0; s < nss; ++s)
      for (int f = 0; f < nf; ++f)
        for (int ca = 0; ca < 2; ++ca) {
          long long o = m.blk_off[((size_t)s * nf + f) * 2 + ca];
          if (o < 0) continue;
          int t = m.connect[((size_t)s * nf + f) * 2 + ca];
          int n1 = m.sst_n[s], n2 = m.sst_n[t];
          for (int j = 0; j < n1; ++j)
            for (int i = 0; i < n2; ++i) {
              double x = m.blk[o + (size_t)j * n2 + i];
              if (x == 0.0) continue;
              size_t idx = (size_t)(2 * f + ca) * ns + m.sst_off[s] + j;
              m.mono_tgt[idx] = m.sst_off[t] + i;
              m.mono_lv[idx] = std::log(std::fabs(x));
              m.mono_neg[idx] = x < 0 ? 1 : 0;
            }
        }
  }
  // dense density-matrix block offsets
  m.dm_off.resize(nss);
  long long acc = 0;
  for (int s = 0; s < nss; ++s) {
    m.dm_off[s] = acc;
    acc += (long long)m.sst_n[s] * m.sst_n[s];
  }
  m.dm_size = acc;
  return true;
}

void direction_blocks(const HostModel& m, int np, const double* dumat, const double* dmuimp,
                      std::vector<double>& out) {
  const int nd = m.nd, nf = m.nf, ns = m.ns, nss = m.nss;
  out.assign((size_t)np * m.dm_size, 0.0);
  // occupation basis: global index of each Fock state, its superstate
  std::vector<int> idx_of(ns, -1), sst_of(ns, -1);
  for (int s = 0; s < nss; ++s)
    for (int i = 0; i < m.sst_n[s]; ++i) {
      idx_of[m.occ_fock[m.sst_off[s] + i]] = m.sst_off[s] + i;
      sst_of[m.occ_fock[m.sst_off[s] + i]] = s;
    }
  auto bit_of = [&](int fl) { return (fl / 2) + nd * (fl % 2); };
  for (int p = 0; p < np; ++p) {
    // D in the occupation basis, superstate blocks (entries leaving a block
    // are dropped, as for H)
    std::vector<std::vector<double>> D(nss);
    for (int s = 0; s < nss; ++s) D[s].assign((size_t)m.sst_n[s] * m.sst_n[s], 0.0);
    auto add = [&](int from, int to, double v) {
      const int s = sst_of[from];
      if (sst_of[to] != s) return;
      const int n = m.sst_n[s];
      D[s][(size_t)(idx_of[from] - m.sst_off[s]) * n + (idx_of[to] - m.sst_off[s])] += v;
    };
    if (dmuimp) {
      const double* mu = dmuimp + (size_t)p * nf * nf;
      for (int f1 = 0; f1 < nf; ++f1)
        for (int f2 = 0; f2 < nf; ++f2) {
          const int b1 = f1 / 2, s1 = f1 % 2, b2 = f2 / 2, s2 = f2 % 2;
          const double v = mu[b1 + nd * (s1 + 2 * (b2 + nd * s2))];
          if (v == 0.0) continue;
          for (int st = 0; st < ns; ++st) {
            double sg = 1.0;
            const int a = apply_op(st, bit_of(f2), true, sg);
            if (a < 0) continue;
            const int c = apply_op(a, bit_of(f1), false, sg);
            if (c < 0) continue;
            add(st, c, v * sg);
          }
        }
    }
    if (dumat) {
      const double* um = dumat + (size_t)p * nf * nf * nf * nf;
      for (int i = 0; i < nf; ++i)
        for (int j = 0; j < nf; ++j)
          for (int k = 0; k < nf; ++k)
            for (int l = 0; l < nf; ++l) {
              const double u = um[i + nf * (j + nf * (k + nf * l))];
              if (u == 0.0) continue;
              for (int st = 0; st < ns; ++st) {
                double sg = 1.0;
                int x = apply_op(st, bit_of(k), true, sg);
                if (x < 0) continue;
                x = apply_op(x, bit_of(l), true, sg);
                if (x < 0) continue;
                x = apply_op(x, bit_of(j), false, sg);
                if (x < 0) continue;
                x = apply_op(x, bit_of(i), false, sg);
                if (x < 0) continue;
                add(st, x, 0.5 * u * sg);
              }
            }
    }
    // rotate into the eigenbasis: V^T D V (D symmetrised like H)
    for (int s = 0; s < nss; ++s) {
      const int n = m.sst_n[s];
      const double* V = m.evec.data() + m.evec_off[s];
      std::vector<double>& d = D[s];
      for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
          const double a = 0.5 * (d[(size_t)j * n + i] + d[(size_t)i * n + j]);
          d[(size_t)j * n + i] = d[(size_t)i * n + j] = a;
        }
      std::vector<double> DV((size_t)n * n, 0.0);
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) {
          const double v = V[(size_t)j * n + k];
          if (v == 0.0) continue;
          for (int i = 0; i < n; ++i) DV[(size_t)j * n + i] += d[(size_t)k * n + i] * v;
        }
      double* o = out.data() + (size_t)p * m.dm_size + m.dm_off[s];
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double acc = 0.0;
          for (int k = 0; k < n; ++k) acc += V[(size_t)i * n + k] * DV[(size_t)j * n + k];
          o[(size_t)j * n + i] = acc;
        }
    }
  }
}

// Normalised empty-trace weights per superstate (init_Trace's choice of the
// outer superstate, Trace.F90:611-669): sum_i exp(-(E_i - Egs) beta)
// accumulated in log form over the states of each superstate.
void empty_trace_weights(const HostModel& m, double beta, std::vector<double>& w) {
  w.assign(m.nss, 0.0);
  double sum = 0;
  for (int s = 0; s < m.nss; ++s) {
    double lg = -1.7976931348623157e308, sg = 0.0;
    double e0 = m.eval[m.sst_off[s]];
    for (int i = 0; i < m.sst_n[s]; ++i) {
      double l = -(e0 - m.egs) * beta - (m.eval[m.sst_off[s] + i] - e0) * beta;
      if (lg >= l) {
        lg = lg + std::log(1.0 + sg * 1.0 * std::exp(l - lg));
      } else {
        lg = l + std::log(1.0 + sg * 1.0 * std::exp(lg - l));
        sg = 1.0;
      }
    }
    w[s] = sg * std::exp(lg);
    sum += w[s];
  }
  for (int s = 0; s < m.nss; ++s) w[s] = w[s] / sum;
}

}  // namespace cthyb
