// Operator allocation and the update compiler. Each emit_* function below records the
// contractions of one reference routine; the reference file:line it follows is named in
// front of it. Phases are written with the same integer expressions as the reference:
//   ph(x)  = (-1)^(x/2)            ((((x)/2)%2)!=0)?-1:1
//   podd(x)= (-1)^x                (((x)%2)!=0)?-1:1
#include "operators.hpp"

#include <unordered_map>

#include <cmath>
#include <cstdlib>
#include <stdexcept>

#include "symm.hpp"

namespace c2g {

using CheMPS2::Problem;
using CheMPS2::SyBookkeeper;

namespace {

inline int ph(int x) { return phase(x); }
inline int podd(int x) { return ((x % 2) != 0) ? -1 : 1; }
inline int64_t align4(int64_t x) { return (x + 3) & ~int64_t(3); }
const Blk kNone;

OpT make_op(BoundaryOps& ops, int boundary, int two_j, int n_elec, int irrep, bool prime_last,
            bool jw, int64_t& off) {
  OpT t;
  t.lay = ops.layouts->get(boundary, two_j, n_elec, irrep);
  t.base = make_ref(ops.slot, off);
  t.moving_right = ops.moving_right;
  t.prime_last = prime_last;
  t.jw_phase = jw;
  off = align4(off + t.lay->size());
  return t;
}

}  // namespace

const OpT& BoundaryOps::Lop(int site) const {
  const int cnt2 = moving_right ? index - site : site - index - 1;
  if (cnt2 < 0 || cnt2 >= static_cast<int>(L.size())) throw std::logic_error("Lop: site out of range");
  return L[cnt2];
}

const OpT& BoundaryOps::Qop(int site) const {
  const int cnt2 = moving_right ? site - index - 1 : index - site;
  if (cnt2 < 0 || cnt2 >= static_cast<int>(Q.size())) throw std::logic_error("Qop: site out of range");
  return Q[cnt2];
}

// CheMPS2/DMRGoperators.cpp:909-1145 (allocateTensors)
void allocate_ops(BoundaryOps& ops, const SyBookkeeper& bk, int L, int index, bool mr, int slot) {
  ops.index = index;
  ops.moving_right = mr;
  ops.slot = slot;
  ops.layouts = std::make_unique<OpLayoutCache>(&bk);
  const int b = index + 1;
  int64_t off = 0;
  auto ir = [&](int s) { return bk.gIrrep(s); };
  const int nleft = mr ? index + 1 : L - 1 - index;   // operators on the swept side
  const int nright = mr ? L - 1 - index : index + 1;  // complementary side
  ops.L.clear();
  for (int c2 = 0; c2 < nleft; c2++) {
    const int site = mr ? index - c2 : index + 1 + c2;
    ops.L.push_back(make_op(ops, b, 1, 1, ir(site), true, true, off));
  }
  ops.F0.assign(nleft, {}); ops.F1.assign(nleft, {}); ops.S0.assign(nleft, {}); ops.S1.assign(nleft, {});
  for (int c2 = 0; c2 < nleft; c2++) {
    for (int c3 = 0; c3 < nleft - c2; c3++) {
      const int s1 = mr ? index - c2 - c3 : index + 1 + c3;
      const int s2 = mr ? index - c3 : index + 1 + c2 + c3;
      const int ip = irrep_prod(ir(s1), ir(s2));
      ops.F0[c2].push_back(make_op(ops, b, 0, 0, ip, true, false, off));
      ops.F1[c2].push_back(make_op(ops, b, 2, 0, ip, mr, false, off));
      ops.S0[c2].push_back(make_op(ops, b, 0, 2, ip, true, false, off));
      if (c2 > 0) ops.S1[c2].push_back(make_op(ops, b, 2, 2, ip, true, false, off));
    }
  }
  ops.A.assign(nright, {}); ops.B.assign(nright, {}); ops.C.assign(nright, {}); ops.D.assign(nright, {});
  for (int c2 = 0; c2 < nright; c2++) {
    for (int c3 = 0; c3 < nright - c2; c3++) {
      const int s1 = mr ? index + 1 + c3 : index - c2 - c3;
      const int s2 = mr ? index + 1 + c2 + c3 : index - c3;
      const int id = irrep_prod(ir(s2), ir(s1));
      ops.A[c2].push_back(make_op(ops, b, 0, 2, id, true, false, off));
      if (c2 > 0) ops.B[c2].push_back(make_op(ops, b, 2, 2, id, true, false, off));
      ops.C[c2].push_back(make_op(ops, b, 0, 0, id, true, false, off));
      ops.D[c2].push_back(make_op(ops, b, 2, 0, id, mr, false, off));
    }
  }
  ops.Q.clear();
  for (int c2 = 0; c2 < nright; c2++) {
    const int site = mr ? index + 1 + c2 : index - c2;
    OpT q = make_op(ops, b, 1, 1, ir(site), true, true, off);
    q.site = site;
    ops.Q.push_back(q);
  }
  ops.X = make_op(ops, b, 0, 0, 0, true, false, off);
  ops.size = off;
  ops.all.clear();
  for (auto& t : ops.L) ops.all.push_back(&t);
  for (auto* v : {&ops.F0, &ops.F1, &ops.S0, &ops.S1, &ops.A, &ops.B, &ops.C, &ops.D})
    for (auto& row : *v)
      for (auto& t : row) ops.all.push_back(&t);
  for (auto& t : ops.Q) ops.all.push_back(&t);
  ops.all.push_back(&ops.X);
}

namespace {

struct Emit {
  TaskBuilder& tb;
  const SyBookkeeper& bk;
  const Problem& prob;
  const MpsT& T;
  int L;
  int shard = 0, nshards = 1;
  const std::unordered_map<Ref, int>* tensor_id = nullptr;
  bool mine(const OpT& o) const {
    if (nshards <= 1) return true;
    return tensor_id->at(o.base) % nshards == shard;
  }

  int dim(int b, int n, int s, int i) const { return bk.gCurrentDim(b, n, s, i); }
  Blk need(const Blk& x) const {
    if (!x.valid) throw std::logic_error("update compiler: a block the reference dereferences is absent");
    return x;
  }
  double V(int a, int b, int c, int d) const { return prob.gMxElement(a, b, c, d); }

  // ---------------------------------------------------------------------------------
  // CheMPS2/TensorOperator.cpp:163-291 (update_moving_right) and :293-405 (moving_left)
  void generic_update(const OpT& out, const OpT& prev) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    const int tj = lay.two_j;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      tb.declare_output(ob);
      const int nu = lay.n_up[ik], nd = nu + lay.n_elec;
      const int su = lay.spin_up[ik], sd = lay.spin_down[ik];
      const int iu = lay.irrep_up[ik], idn = irrep_prod(iu, lay.n_irrep);
      for (int geval = 0; geval < 6; geval++) {
        int n2u, n2d, s2u, s2d, i2u, i2d;
        const int dn = out.moving_right ? -1 : +1;  // direction to the previous boundary
        const int site = out.moving_right ? index - 1 : index;
        switch (geval) {
          case 0: s2u = su; s2d = sd; n2u = nu; n2d = nd; i2u = iu; i2d = idn; break;
          case 1: s2u = su; s2d = sd; n2u = nu + 2 * dn; n2d = nd + 2 * dn; i2u = iu; i2d = idn; break;
          case 2: s2u = su - 1; s2d = sd - 1; n2u = nu + dn; n2d = nd + dn;
                  i2u = irrep_prod(iu, bk.gIrrep(site)); i2d = irrep_prod(idn, bk.gIrrep(site)); break;
          case 3: s2u = su - 1; s2d = sd + 1; n2u = nu + dn; n2d = nd + dn;
                  i2u = irrep_prod(iu, bk.gIrrep(site)); i2d = irrep_prod(idn, bk.gIrrep(site)); break;
          case 4: s2u = su + 1; s2d = sd - 1; n2u = nu + dn; n2d = nd + dn;
                  i2u = irrep_prod(iu, bk.gIrrep(site)); i2d = irrep_prod(idn, bk.gIrrep(site)); break;
          default: s2u = su + 1; s2d = sd + 1; n2u = nu + dn; n2d = nd + dn;
                  i2u = irrep_prod(iu, bk.gIrrep(site)); i2d = irrep_prod(idn, bk.gIrrep(site)); break;
        }
        if (std::abs(s2u - s2d) > tj) continue;
        const int pb = out.moving_right ? index - 1 : index + 1;
        if (dim(pb, n2u, s2u, i2u) <= 0 || dim(pb, n2d, s2d, i2d) <= 0) continue;
        double alpha = 1.0;
        const int jw3 = out.jw_phase ? 3 : 1;
        if (out.moving_right) {
          // labels: left = previous boundary (2), right = this boundary
          const int slu = s2u, sld = s2d, sru = su, srd = sd;
          if (geval >= 2) {
            if (tj == 0) {
              alpha = out.jw_phase ? -1.0 : 1.0;
            } else if (out.prime_last) {
              alpha = ph(sru + sld + tj + jw3) * std::sqrt((sld + 1.0) * (sru + 1.0)) *
                      wigner6j(slu, sld, tj, srd, sru, 1);
            } else {
              alpha = ph(srd + slu + tj + jw3) * std::sqrt((slu + 1.0) * (srd + 1.0)) *
                      wigner6j(sld, slu, tj, sru, srd, 1);
            }
          }
          const Blk Tu = need(T.blk(n2u, s2u, i2u, nu, su, iu));
          const Blk Td = need(T.blk(n2d, s2d, i2d, nd, sd, idn));
          const Blk Pb = need(prev.blk(n2u, s2u, i2u, n2d, s2d, i2d));
          tb.contract(ob, alpha, Tu, true, Pb, false, Td, false);
        } else {
          const int slu = su, sld = sd, sru = s2u, srd = s2d;
          if (geval >= 2) {
            if (tj == 0) {
              alpha = (out.jw_phase ? -1.0 : 1.0) * ((sru + 1.0) / (slu + 1));
            } else if (out.prime_last) {
              alpha = ph(sru + sld + tj + jw3) * (srd + 1) * std::sqrt((sru + 1.0) / (sld + 1)) *
                      wigner6j(sru, srd, tj, sld, slu, 1);
            } else {
              alpha = ph(srd + slu + tj + jw3) * (sru + 1) * std::sqrt((srd + 1.0) / (slu + 1)) *
                      wigner6j(srd, sru, tj, slu, sld, 1);
            }
          }
          const Blk Tu = need(T.blk(nu, su, iu, n2u, s2u, i2u));
          const Blk Td = need(T.blk(nd, sd, idn, n2d, s2d, i2d));
          const Blk Pb = need(prev.blk(n2u, s2u, i2u, n2d, s2d, i2d));
          tb.contract(ob, alpha, Tu, false, Pb, false, Td, true);
        }
      }
    }
  }

  void declare_all(const OpT& out) {
    if (!mine(out)) return;
    for (int ik = 0; ik < out.lay->nkappa; ik++) tb.declare_output(out.blk_k(ik));
  }

  // ---------------------------------------------------------------------------------
  // CheMPS2/TensorL.cpp:57-135 (create_right / create_left without a previous tensor)
  void L_create(const OpT& out) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      tb.declare_output(ob);
      const int nu = lay.n_up[ik], nd = nu + 1;
      const int iu = lay.irrep_up[ik], idn = irrep_prod(iu, lay.n_irrep);
      const int su = lay.spin_up[ik], sd = lay.spin_down[ik];
      for (int geval = 0; geval < 2; geval++) {
        if (out.moving_right) {
          int nl, sl, il;
          if (geval == 0) { nl = nu; sl = su; il = iu; } else { nl = nu - 1; sl = sd; il = idn; }
          if (dim(index - 1, nl, sl, il) <= 0) continue;
          const double alpha = (geval == 1) ? ph(sd - su + 1) * std::sqrt((su + 1.0) / (sd + 1)) : 1.0;
          tb.contract(ob, alpha, need(T.blk(nl, sl, il, nu, su, iu)), true,
                      need(T.blk(nl, sl, il, nd, sd, idn)), false, kNone, false);
        } else {
          int nr, sr, irr;
          if (geval == 0) { nr = nd; sr = sd; irr = idn; } else { nr = nu + 2; sr = su; irr = iu; }
          if (dim(index + 1, nr, sr, irr) <= 0) continue;
          const double alpha = (geval == 1) ? ph(su - sd + 1) * std::sqrt((su + 1.0) / (sd + 1)) : 1.0;
          tb.contract(ob, alpha, kNone, false, need(T.blk(nu, su, iu, nr, sr, irr)), false,
                      need(T.blk(nd, sd, idn, nr, sr, irr)), true);
        }
      }
    }
  }

  // ---------------------------------------------------------------------------------
  // CheMPS2/TensorF0.cpp:53-138 (makenewRight/Left from the MPS only)
  void F0_new(const OpT& out) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    const double sqrt2 = std::sqrt(2.0);
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      tb.declare_output(ob);
      const int n = lay.n_up[ik], s = lay.spin_up[ik], i = lay.irrep_up[ik];
      for (int geval = 0; geval < 3; geval++) {
        if (out.moving_right) {
          int nl, sl, il;
          if (geval == 0) { nl = n - 2; sl = s; il = i; }
          else if (geval == 1) { nl = n - 1; sl = s - 1; il = irrep_prod(i, bk.gIrrep(index - 1)); }
          else { nl = n - 1; sl = s + 1; il = irrep_prod(i, bk.gIrrep(index - 1)); }
          if (dim(index - 1, nl, sl, il) <= 0) continue;
          const Blk Tb = need(T.blk(nl, sl, il, n, s, i));
          const double alpha = (geval == 0) ? sqrt2 : (0.5 * sqrt2);
          tb.contract(ob, alpha, Tb, true, Tb, false, kNone, false);
        } else {
          int nr, sr, irr;
          if (geval == 0) { nr = n + 2; sr = s; irr = i; }
          else if (geval == 1) { nr = n + 1; sr = s - 1; irr = irrep_prod(i, bk.gIrrep(index)); }
          else { nr = n + 1; sr = s + 1; irr = irrep_prod(i, bk.gIrrep(index)); }
          if (dim(index + 1, nr, sr, irr) <= 0) continue;
          const Blk Tb = need(T.blk(n, s, i, nr, sr, irr));
          double alpha = sqrt2;
          if (geval >= 1) alpha *= 0.5 * (sr + 1.0) / (s + 1.0);
          tb.contract(ob, alpha, kNone, false, Tb, false, Tb, true);
        }
      }
    }
  }

  // CheMPS2/TensorF1.cpp:54-118
  void F1_new(const OpT& out) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      tb.declare_output(ob);
      const int n = lay.n_up[ik], su = lay.spin_up[ik], sd = lay.spin_down[ik], i = lay.irrep_up[ik];
      for (int geval = 0; geval < 2; geval++) {
        const int sx = su + ((geval == 0) ? -1 : 1);
        if (sx < 0 || std::abs(sd - sx) >= 2) continue;
        if (out.moving_right) {
          const int il = irrep_prod(i, bk.gIrrep(index - 1));
          if (dim(index - 1, n - 1, sx, il) <= 0) continue;
          const double alpha = ph(sx + sd + 3) * std::sqrt(3.0 * (su + 1)) * wigner6j(1, 1, 2, su, sd, sx);
          tb.contract(ob, alpha, need(T.blk(n - 1, sx, il, n, su, i)), true,
                      need(T.blk(n - 1, sx, il, n, sd, i)), false, kNone, false);
        } else {
          const int irr = irrep_prod(i, bk.gIrrep(index));
          if (dim(index + 1, n + 1, sx, irr) <= 0) continue;
          const double alpha = ph(sd + sx + 1) * std::sqrt(3.0 / (su + 1.0)) * (sx + 1) *
                               wigner6j(1, 1, 2, su, sd, sx);
          tb.contract(ob, alpha, kNone, false, need(T.blk(n, su, i, n + 1, sx, irr)), false,
                      need(T.blk(n, sd, i, n + 1, sx, irr)), true);
        }
      }
    }
  }

  // CheMPS2/TensorS0.cpp:53-99
  void S0_new(const OpT& out) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      tb.declare_output(ob);
      const int n = lay.n_up[ik], s = lay.spin_up[ik], i = lay.irrep_up[ik];
      if (out.moving_right) {
        if (dim(index - 1, n, s, i) <= 0) continue;
        tb.contract(ob, std::sqrt(2.0), need(T.blk(n, s, i, n, s, i)), true,
                    need(T.blk(n, s, i, n + 2, s, i)), false, kNone, false);
      } else {
        if (dim(index + 1, n + 2, s, i) <= 0) continue;
        tb.contract(ob, std::sqrt(2.0), kNone, false, need(T.blk(n, s, i, n + 2, s, i)), false,
                    need(T.blk(n + 2, s, i, n + 2, s, i)), true);
      }
    }
  }

  // Shared driver of the makenew(L, T) routines of F0, F1, S0 and S1: four "geval"
  // cases, each a sandwich  out += alpha * Tup^T * Lblk * Tdown  (moving right) or
  // out += alpha * Tup * Lblk * Tdown^T (moving left).
  template <class Cases>
  void makenew_L(const OpT& out, const OpT& Lop, Cases cases) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      tb.declare_output(ob);
      const int n = lay.n_up[ik], su = lay.spin_up[ik], sd = lay.spin_down[ik], i = lay.irrep_up[ik];
      const int idn = irrep_prod(lay.n_irrep, i);
      const int nd = n + lay.n_elec;
      for (int geval = 0; geval < 4; geval++) {
        int nx, sxu, ixu, sxd, ixd;  // previous-boundary sectors: up (nx) and down (nx + 1)
        double alpha;
        bool spin_check;
        if (!cases(geval, n, su, sd, i, idn, nx, sxu, ixu, sxd, ixd, alpha, spin_check)) continue;
        const int pb = out.moving_right ? index - 1 : index + 1;
        if (dim(pb, nx, sxu, ixu) <= 0 || dim(pb, nx + 1, sxd, ixd) <= 0) continue;
        if (spin_check && std::abs(sxu - sxd) >= 2) continue;
        const Blk Lb = need(Lop.blk(nx, sxu, ixu, nx + 1, sxd, ixd));
        if (out.moving_right) {
          tb.contract(ob, alpha, need(T.blk(nx, sxu, ixu, n, su, i)), true, Lb, false,
                      need(T.blk(nx + 1, sxd, ixd, nd, sd, idn)), false);
        } else {
          tb.contract(ob, alpha, need(T.blk(n, su, i, nx, sxu, ixu)), false, Lb, false,
                      need(T.blk(nd, sd, idn, nx + 1, sxd, ixd)), true);
        }
      }
    }
  }

  // CheMPS2/TensorF0.cpp:140-211 (right) and :213-285 (left)
  void F0_newL(const OpT& out, const OpT& Lop) {
    if (!mine(out)) return;
    const int index = out.lay->index;
    const bool mr = out.moving_right;
    const int Li = Lop.irrep();
    makenew_L(out, Lop, [&](int g, int n, int su, int sd, int i, int idn, int& nx, int& sxu, int& ixu,
                            int& sxd, int& ixd, double& alpha, bool& sc) {
      (void)sd;
      sc = false;
      if (mr) {
        const int il = irrep_prod(i, bk.gIrrep(index - 1));
        switch (g) {
          case 0: nx = n - 1; sxu = su - 1; ixu = il; sxd = su; ixd = idn; break;
          case 1: nx = n - 1; sxu = su + 1; ixu = il; sxd = su; ixd = idn; break;
          case 2: nx = n - 2; sxu = su; ixu = i; sxd = su - 1; ixd = irrep_prod(i, Li); break;
          default: nx = n - 2; sxu = su; ixu = i; sxd = su + 1; ixd = irrep_prod(i, Li); break;
        }
        if (sxu < 0 || sxd < 0) return false;
        alpha = (g <= 1) ? std::sqrt(0.5) : ph(su + 1 - sxd) * std::sqrt(0.5 * (sxd + 1.0) / (su + 1.0));
      } else {
        const int irr = irrep_prod(i, bk.gIrrep(index));
        switch (g) {
          case 0: nx = n; sxu = su; ixu = i; sxd = su - 1; ixd = irrep_prod(i, Li); break;
          case 1: nx = n; sxu = su; ixu = i; sxd = su + 1; ixd = irrep_prod(i, Li); break;
          case 2: nx = n + 1; sxu = su - 1; ixu = irr; sxd = su; ixd = idn; break;
          default: nx = n + 1; sxu = su + 1; ixu = irr; sxd = su; ixd = idn; break;
        }
        if (sxu < 0 || sxd < 0) return false;
        alpha = (g <= 1) ? std::sqrt(0.5) * (sxd + 1.0) / (su + 1.0)
                         : ph(su - sxu + 1) * std::sqrt(0.5 * (sxu + 1.0) / (su + 1.0));
      }
      return true;
    });
  }

  // CheMPS2/TensorF1.cpp:120-192 (right) and :194-269 (left)
  void F1_newL(const OpT& out, const OpT& Lop) {
    if (!mine(out)) return;
    const int index = out.lay->index;
    const bool mr = out.moving_right;
    const int Li = Lop.irrep();
    makenew_L(out, Lop, [&](int g, int n, int su, int sd, int i, int idn, int& nx, int& sxu, int& ixu,
                            int& sxd, int& ixd, double& alpha, bool& sc) {
      sc = true;
      if (mr) {
        const int il = irrep_prod(i, bk.gIrrep(index - 1));
        switch (g) {
          case 0: nx = n - 1; sxu = su - 1; ixu = il; sxd = sd; ixd = idn; break;
          case 1: nx = n - 1; sxu = su + 1; ixu = il; sxd = sd; ixd = idn; break;
          case 2: nx = n - 2; sxu = su; ixu = i; sxd = sd - 1; ixd = irrep_prod(i, Li); break;
          default: nx = n - 2; sxu = su; ixu = i; sxd = sd + 1; ixd = irrep_prod(i, Li); break;
        }
        if (sxu < 0 || sxd < 0) return false;
        if (g <= 1) alpha = ph(sxu + sd + 3) * std::sqrt(3.0 * (su + 1)) * wigner6j(1, 1, 2, su, sd, sxu);
        else alpha = ph(su + sd + 2) * std::sqrt(3.0 * (sxd + 1)) * wigner6j(1, 1, 2, su, sd, sxd);
      } else {
        const int irr = irrep_prod(i, bk.gIrrep(index));
        switch (g) {
          case 0: nx = n; sxu = su; ixu = i; sxd = sd - 1; ixd = irrep_prod(i, Li); break;
          case 1: nx = n; sxu = su; ixu = i; sxd = sd + 1; ixd = irrep_prod(i, Li); break;
          case 2: nx = n + 1; sxu = su - 1; ixu = irr; sxd = sd; ixd = idn; break;
          default: nx = n + 1; sxu = su + 1; ixu = irr; sxd = sd; ixd = idn; break;
        }
        if (sxu < 0 || sxd < 0) return false;
        if (g <= 1)
          alpha = ph(sd + sxd + 1) * std::sqrt(3.0 / (su + 1.0)) * (sxd + 1) * wigner6j(1, 1, 2, su, sd, sxd);
        else
          alpha = podd(su) * std::sqrt(3.0 * (sxu + 1.0) * (sd + 1.0) / (su + 1.0)) *
                  wigner6j(1, 1, 2, su, sd, sxu);
      }
      return true;
    });
  }

  // CheMPS2/TensorS0.cpp:101-172 (right) and :174-246 (left)
  void S0_newL(const OpT& out, const OpT& Lop) {
    if (!mine(out)) return;
    const int index = out.lay->index;
    const bool mr = out.moving_right;
    const int Li = Lop.irrep();
    makenew_L(out, Lop, [&](int g, int n, int su, int sd, int i, int idn, int& nx, int& sxu, int& ixu,
                            int& sxd, int& ixd, double& alpha, bool& sc) {
      (void)sd;
      sc = false;
      if (mr) {
        const int il = irrep_prod(i, bk.gIrrep(index - 1));
        switch (g) {
          case 0: nx = n; sxu = su; ixu = i; sxd = su - 1; ixd = irrep_prod(i, Li); break;
          case 1: nx = n; sxu = su; ixu = i; sxd = su + 1; ixd = irrep_prod(i, Li); break;
          case 2: nx = n - 1; sxu = su - 1; ixu = il; sxd = su; ixd = idn; break;
          default: nx = n - 1; sxu = su + 1; ixu = il; sxd = su; ixd = idn; break;
        }
        if (sxu < 0 || sxd < 0) return false;
        alpha = (g <= 1) ? ph(su - sxd + 1) * std::sqrt(0.5 * (sxd + 1.0) / (su + 1.0)) : -std::sqrt(0.5);
      } else {
        const int irr = irrep_prod(i, bk.gIrrep(index));
        switch (g) {
          case 0: nx = n + 1; sxu = su - 1; ixu = irr; sxd = su; ixd = idn; break;
          case 1: nx = n + 1; sxu = su + 1; ixu = irr; sxd = su; ixd = idn; break;
          case 2: nx = n + 2; sxu = su; ixu = i; sxd = su - 1; ixd = irrep_prod(i, Li); break;
          default: nx = n + 2; sxu = su; ixu = i; sxd = su + 1; ixd = irrep_prod(i, Li); break;
        }
        if (sxu < 0 || sxd < 0) return false;
        alpha = (g <= 1) ? ph(su - sxu + 1) * std::sqrt(0.5 * (sxu + 1.0) / (su + 1.0))
                         : -std::sqrt(0.5) * (sxd + 1.0) / (su + 1.0);
      }
      return true;
    });
  }

  // CheMPS2/TensorS1.cpp:47-119 (right) and :121-195 (left)
  void S1_newL(const OpT& out, const OpT& Lop) {
    if (!mine(out)) return;
    const int index = out.lay->index;
    const bool mr = out.moving_right;
    const int Li = Lop.irrep();
    makenew_L(out, Lop, [&](int g, int n, int su, int sd, int i, int idn, int& nx, int& sxu, int& ixu,
                            int& sxd, int& ixd, double& alpha, bool& sc) {
      sc = true;
      if (mr) {
        const int il = irrep_prod(i, bk.gIrrep(index - 1));
        switch (g) {
          case 0: nx = n; sxu = su; ixu = i; sxd = sd - 1; ixd = irrep_prod(i, Li); break;
          case 1: nx = n; sxu = su; ixu = i; sxd = sd + 1; ixd = irrep_prod(i, Li); break;
          case 2: nx = n - 1; sxu = su - 1; ixu = il; sxd = sd; ixd = idn; break;
          default: nx = n - 1; sxu = su + 1; ixu = il; sxd = sd; ixd = idn; break;
        }
        if (sxu < 0 || sxd < 0) return false;
        if (g <= 1) alpha = ph(su + sd + 2) * std::sqrt(3.0 * (sxd + 1)) * wigner6j(1, 1, 2, su, sd, sxd);
        else alpha = ph(sxu + sd + 1) * std::sqrt(3.0 * (su + 1)) * wigner6j(1, 1, 2, su, sd, sxu);
      } else {
        const int irr = irrep_prod(i, bk.gIrrep(index));
        switch (g) {
          case 0: nx = n + 1; sxu = su - 1; ixu = irr; sxd = sd; ixd = idn; break;
          case 1: nx = n + 1; sxu = su + 1; ixu = irr; sxd = sd; ixd = idn; break;
          case 2: nx = n + 2; sxu = su; ixu = i; sxd = sd - 1; ixd = irrep_prod(i, Li); break;
          default: nx = n + 2; sxu = su; ixu = i; sxd = sd + 1; ixd = irrep_prod(i, Li); break;
        }
        if (sxu < 0 || sxd < 0) return false;
        if (g <= 1) alpha = ph(su + sd + 2) * std::sqrt(3.0 * (sxu + 1)) * wigner6j(1, 1, 2, su, sd, sxu);
        else
          alpha = ph(su + sxd + 1) * std::sqrt(3.0 / (sd + 1.0)) * (sxd + 1) * wigner6j(1, 1, 2, su, sd, sxd);
      }
      return true;
    });
  }

  // ---------------------------------------------------------------------------------
  // CheMPS2/TensorQ.cpp:45-104 (AddTermSimple)
  void Q_simple(const OpT& out, int mps_site) {
    if (!mine(out)) return;
    if (bk.gIrrep(mps_site) != out.irrep()) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    const int site = out.site;
    const double mx = out.moving_right ? V(index - 1, index - 1, index - 1, site) : V(site, index, index, index);
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      const int n = lay.n_up[ik], su = lay.spin_up[ik], sd = lay.spin_down[ik], i = lay.irrep_up[ik];
      const int id = irrep_prod(out.irrep(), i);
      if (out.moving_right) {
        if (dim(index - 1, n - 1, sd, id) <= 0) continue;
        const double alpha = ph(sd + 1 - su) * mx * std::sqrt((su + 1.0) / (sd + 1.0));
        tb.contract(ob, alpha, need(T.blk(n - 1, sd, id, n, su, i)), true,
                    need(T.blk(n - 1, sd, id, n + 1, sd, id)), false, kNone, false);
      } else {
        if (dim(index + 1, n + 2, su, i) <= 0) continue;
        const double alpha = ph(su + 1 - sd) * mx * std::sqrt((su + 1.0) / (sd + 1.0));
        tb.contract(ob, alpha, kNone, false, need(T.blk(n, su, i, n + 2, su, i)), false,
                    need(T.blk(n + 1, sd, id, n + 2, su, i)), true);
      }
    }
  }

  // CheMPS2/TensorQ.cpp:106-384 (AddTermsL). `Lprev(site)` is the creator on `site` at
  // the previous boundary.
  template <class LF>
  void Q_L(const OpT& out, LF Lprev) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    const int site = out.site;
    const int nirr = out.irrep();
    std::vector<int> locs;
    if (out.moving_right) {
      for (int loca = 0; loca < index - 1; loca++)
        if (Lprev(loca).irrep() == nirr) locs.push_back(loca);
    } else {
      for (int loca = index + 1; loca < L; loca++)
        if (Lprev(loca).irrep() == nirr) locs.push_back(loca);
    }
    if (locs.empty()) return;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      const int n = lay.n_up[ik], su = lay.spin_up[ik], sd = lay.spin_down[ik], i = lay.irrep_up[ik];
      const int id = irrep_prod(i, nirr);
      if (out.moving_right) {
        // case 1
        if (dim(index - 1, n, su, i) > 0 && dim(index - 1, n - 1, sd, id) > 0) {
          thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
          parts.clear();
          for (int loca : locs)
            parts.push_back({V(loca, site, index - 1, index - 1), need(Lprev(loca).blk(n - 1, sd, id, n, su, i))});
          const Blk W = tb.combine(parts, dim(index - 1, n - 1, sd, id), dim(index - 1, n, su, i));
          const double alpha = ph(sd + 1 - su) * std::sqrt((su + 1.0) / (sd + 1.0));
          tb.contract(ob, alpha, need(T.blk(n, su, i, n, su, i)), true, W, true,
                      need(T.blk(n - 1, sd, id, n + 1, sd, id)), false);
        }
        // case 2
        if (dim(index - 1, n - 2, su, i) > 0 && dim(index - 1, n - 1, sd, id) > 0) {
          thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
          parts.clear();
          for (int loca : locs)
            parts.push_back({2 * V(loca, index - 1, site, index - 1) - V(loca, index - 1, index - 1, site),
                             need(Lprev(loca).blk(n - 2, su, i, n - 1, sd, id))});
          const Blk W = tb.combine(parts, dim(index - 1, n - 2, su, i), dim(index - 1, n - 1, sd, id));
          tb.contract(ob, 1.0, need(T.blk(n - 2, su, i, n, su, i)), true, W, false,
                      need(T.blk(n - 1, sd, id, n + 1, sd, id)), false);
        }
        // case 3
        for (int slu = su - 1; slu <= su + 1; slu += 2) {
          for (int sld = sd - 1; sld <= sd + 1; sld += 2) {
            if (sld < 0 || slu < 0 || std::abs(sld - slu) >= 2) continue;
            const int ilu = irrep_prod(i, bk.gIrrep(index - 1));
            const int ild = irrep_prod(id, bk.gIrrep(index - 1));
            const int dlu = dim(index - 1, n - 1, slu, ilu), dld = dim(index - 1, n, sld, ild);
            if (dlu <= 0 || dld <= 0) continue;
            const double factor = ph(su + sld) * std::sqrt((sld + 1) * (su + 1.0)) * wigner6j(su, sd, 1, sld, slu, 1);
            thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
            parts.clear();
            for (int loca : locs) {
              double a = factor * V(loca, index - 1, site, index - 1);
              if (sld == su) a += V(loca, index - 1, index - 1, site);
              parts.push_back({a, need(Lprev(loca).blk(n - 1, slu, ilu, n, sld, ild))});
            }
            const Blk W = tb.combine(parts, dlu, dld);
            tb.contract(ob, 1.0, need(T.blk(n - 1, slu, ilu, n, su, i)), true, W, false,
                        need(T.blk(n, sld, ild, n + 1, sd, id)), false);
          }
        }
      } else {
        // case 1
        if (dim(index + 1, n + 2, su, i) > 0 && dim(index + 1, n + 1, sd, id) > 0) {
          thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
          parts.clear();
          for (int loca : locs)
            parts.push_back({V(site, loca, index, index), need(Lprev(loca).blk(n + 1, sd, id, n + 2, su, i))});
          const Blk W = tb.combine(parts, dim(index + 1, n + 1, sd, id), dim(index + 1, n + 2, su, i));
          const double alpha = ph(su + 1 - sd) * std::sqrt((su + 1.0) / (sd + 1.0));
          tb.contract(ob, alpha, need(T.blk(n, su, i, n + 2, su, i)), false, W, true,
                      need(T.blk(n + 1, sd, id, n + 1, sd, id)), true);
        }
        // case 2
        if (dim(index + 1, n + 2, su, i) > 0 && dim(index + 1, n + 3, sd, id) > 0) {
          thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
          parts.clear();
          for (int loca : locs)
            parts.push_back({2 * V(site, index, loca, index) - V(site, index, index, loca),
                             need(Lprev(loca).blk(n + 2, su, i, n + 3, sd, id))});
          const Blk W = tb.combine(parts, dim(index + 1, n + 2, su, i), dim(index + 1, n + 3, sd, id));
          tb.contract(ob, 1.0, need(T.blk(n, su, i, n + 2, su, i)), false, W, false,
                      need(T.blk(n + 1, sd, id, n + 3, sd, id)), true);
        }
        // case 3
        for (int sru = su - 1; sru <= su + 1; sru += 2) {
          for (int srd = sd - 1; srd <= sd + 1; srd += 2) {
            if (srd < 0 || sru < 0 || std::abs(srd - sru) >= 2) continue;
            const int iru = irrep_prod(i, bk.gIrrep(index));
            const int ird = irrep_prod(id, bk.gIrrep(index));
            const int dru = dim(index + 1, n + 1, sru, iru), drd = dim(index + 1, n + 2, srd, ird);
            if (dru <= 0 || drd <= 0) continue;
            const double f1 = ph(sd + sru) * std::sqrt((sru + 1.0) / (sd + 1.0)) * (srd + 1) *
                              wigner6j(su, sd, 1, srd, sru, 1);
            const double f2 = (srd + 1.0) / (sd + 1.0);
            thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
            parts.clear();
            for (int loca : locs) {
              double a = f1 * V(site, index, loca, index);
              if (sru == sd) a += f2 * V(site, index, index, loca);
              parts.push_back({a, need(Lprev(loca).blk(n + 1, sru, iru, n + 2, srd, ird))});
            }
            const Blk W = tb.combine(parts, dru, drd);
            tb.contract(ob, 1.0, need(T.blk(n, su, i, n + 1, sru, iru)), false, W, false,
                        need(T.blk(n + 1, sd, id, n + 2, srd, ird)), true);
          }
        }
      }
    }
  }

  // CheMPS2/TensorQ.cpp:386-599 (AddTermsAB)
  void Q_AB(const OpT& out, const OpT& A, const OpT& B) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      const int n = lay.n_up[ik], su = lay.spin_up[ik], sd = lay.spin_down[ik], i = lay.irrep_up[ik];
      const int id = irrep_prod(i, out.irrep());
      if (out.moving_right) {
        const int ilu = irrep_prod(i, bk.gIrrep(index - 1));
        for (int slu = su - 1; slu <= su + 1; slu += 2) {  // case 1
          const int dlu = dim(index - 1, n - 1, slu, ilu), dld = dim(index - 1, n + 1, sd, id);
          if (dlu <= 0 || dld <= 0) continue;
          const double fB = ph(slu + sd + 2) * std::sqrt(3.0 * (su + 1)) * wigner6j(1, 2, 1, sd, su, slu);
          const Blk Bb = need(B.blk(n - 1, slu, ilu, n + 1, sd, id));
          Blk M;
          double alpha;
          if (slu == sd) {
            const double fA = ph(sd + 1 - su) * std::sqrt(0.5 * (su + 1.0) / (sd + 1.0));
            M = tb.combine({{fA, need(A.blk(n - 1, slu, ilu, n + 1, sd, id))}, {fB, Bb}}, dlu, dld);
            alpha = 1.0;
          } else {
            M = Bb;
            alpha = fB;
          }
          tb.contract(ob, alpha, need(T.blk(n - 1, slu, ilu, n, su, i)), true, M, false,
                      need(T.blk(n + 1, sd, id, n + 1, sd, id)), false);
        }
        const int ild = irrep_prod(id, bk.gIrrep(index - 1));
        for (int sld = sd - 1; sld <= sd + 1; sld += 2) {  // case 2
          const int dlu = dim(index - 1, n - 2, su, i), dld = dim(index - 1, n, sld, ild);
          if (dlu <= 0 || dld <= 0) continue;
          const double fB = ph(su + sd + 1) * std::sqrt(3.0 * (sld + 1)) * wigner6j(1, 2, 1, su, sd, sld);
          const Blk Bb = need(B.blk(n - 2, su, i, n, sld, ild));
          Blk M;
          double alpha;
          if (sld == su) {
            M = tb.combine({{-std::sqrt(0.5), need(A.blk(n - 2, su, i, n, sld, ild))}, {fB, Bb}}, dlu, dld);
            alpha = 1.0;
          } else {
            M = Bb;
            alpha = fB;
          }
          tb.contract(ob, alpha, need(T.blk(n - 2, su, i, n, su, i)), true, M, false,
                      need(T.blk(n, sld, ild, n + 1, sd, id)), false);
        }
      } else {
        const int ird = irrep_prod(id, bk.gIrrep(index));
        for (int srd = sd - 1; srd <= sd + 1; srd += 2) {  // case 1
          const int dru = dim(index + 1, n, su, i), drd = dim(index + 1, n + 2, srd, ird);
          if (dru <= 0 || drd <= 0) continue;
          const double fB = ph(srd + su + 2) * std::sqrt(3.0 / (sd + 1.0)) * (srd + 1) * wigner6j(1, 1, 2, su, srd, sd);
          const Blk Bb = need(B.blk(n, su, i, n + 2, srd, ird));
          Blk M;
          double alpha;
          if (srd == su) {
            const double fA = ph(su + 1 - sd) * std::sqrt(0.5 * (su + 1.0) / (sd + 1.0));
            M = tb.combine({{fA, need(A.blk(n, su, i, n + 2, srd, ird))}, {fB, Bb}}, dru, drd);
            alpha = 1.0;
          } else {
            M = Bb;
            alpha = fB;
          }
          tb.contract(ob, alpha, need(T.blk(n, su, i, n, su, i)), false, M, false,
                      need(T.blk(n + 1, sd, id, n + 2, srd, ird)), true);
        }
        const int iru = irrep_prod(i, bk.gIrrep(index));
        for (int sru = su - 1; sru <= su + 1; sru += 2) {  // case 2
          const int dru = dim(index + 1, n + 1, sru, iru), drd = dim(index + 1, n + 3, sd, id);
          if (dru <= 0 || drd <= 0) continue;
          const double fB = ph(su + sd + 1) * std::sqrt(3.0 * (sru + 1)) * wigner6j(1, 1, 2, sru, sd, su);
          const Blk Bb = need(B.blk(n + 1, sru, iru, n + 3, sd, id));
          Blk M;
          double alpha;
          if (sru == sd) {
            M = tb.combine({{-std::sqrt(0.5), need(A.blk(n + 1, sru, iru, n + 3, sd, id))}, {fB, Bb}}, dru, drd);
            alpha = 1.0;
          } else {
            M = Bb;
            alpha = fB;
          }
          tb.contract(ob, alpha, need(T.blk(n, su, i, n + 1, sru, iru)), false, M, false,
                      need(T.blk(n + 1, sd, id, n + 3, sd, id)), true);
        }
      }
    }
  }

  // CheMPS2/TensorQ.cpp:601-785 (AddTermsCD)
  void Q_CD(const OpT& out, const OpT& C, const OpT& D) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      const int n = lay.n_up[ik], su = lay.spin_up[ik], sd = lay.spin_down[ik], i = lay.irrep_up[ik];
      const int id = irrep_prod(i, out.irrep());
      if (out.moving_right) {
        const int ild = irrep_prod(id, bk.gIrrep(index - 1));
        for (int sld = sd - 1; sld <= sd + 1; sld += 2) {  // case 1
          const int dlu = dim(index - 1, n, su, i), dld = dim(index - 1, n, sld, ild);
          if (dlu <= 0 || dld <= 0) continue;
          const double fD = ph(su + sd + 1) * std::sqrt(3.0 * (sld + 1)) * wigner6j(1, 2, 1, su, sd, sld);
          thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
          parts.assign(1, {fD, need(D.blk(n, su, i, n, sld, ild))});
          if (sld == su) parts.push_back({std::sqrt(0.5), need(C.blk(n, su, i, n, sld, ild))});
          const Blk M = tb.combine(parts, dlu, dld);
          tb.contract(ob, 1.0, need(T.blk(n, su, i, n, su, i)), true, M, false,
                      need(T.blk(n, sld, ild, n + 1, sd, id)), false);
        }
        const int ilu = irrep_prod(i, bk.gIrrep(index - 1));
        for (int slu = su - 1; slu <= su + 1; slu += 2) {  // case 2
          const int dlu = dim(index - 1, n - 1, slu, ilu), dld = dim(index - 1, n - 1, sd, id);
          if (dlu <= 0 || dld <= 0) continue;
          const double fD = ph(slu + sd) * std::sqrt(3.0 * (su + 1)) * wigner6j(1, 2, 1, sd, su, slu);
          thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
          parts.assign(1, {fD, need(D.blk(n - 1, slu, ilu, n - 1, sd, id))});
          if (slu == sd)
            parts.push_back({ph(sd + 1 - su) * std::sqrt(0.5 * (su + 1.0) / (sd + 1.0)),
                             need(C.blk(n - 1, slu, ilu, n - 1, sd, id))});
          const Blk M = tb.combine(parts, dlu, dld);
          tb.contract(ob, 1.0, need(T.blk(n - 1, slu, ilu, n, su, i)), true, M, false,
                      need(T.blk(n - 1, sd, id, n + 1, sd, id)), false);
        }
      } else {
        const int iru = irrep_prod(i, bk.gIrrep(index));
        for (int sru = su - 1; sru <= su + 1; sru += 2) {  // case 1
          const int dru = dim(index + 1, n + 1, sru, iru), drd = dim(index + 1, n + 1, sd, id);
          if (dru <= 0 || drd <= 0) continue;
          const double fD = ph(su + sru + 3) * std::sqrt(3.0 / (sd + 1.0)) * (sru + 1) * wigner6j(1, 1, 2, sru, sd, su);
          thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
          parts.assign(1, {fD, need(D.blk(n + 1, sru, iru, n + 1, sd, id))});
          if (sru == sd) parts.push_back({std::sqrt(0.5), need(C.blk(n + 1, sru, iru, n + 1, sd, id))});
          const Blk M = tb.combine(parts, dru, drd);
          tb.contract(ob, 1.0, need(T.blk(n, su, i, n + 1, sru, iru)), false, M, false,
                      need(T.blk(n + 1, sd, id, n + 1, sd, id)), true);
        }
        const int ird = irrep_prod(id, bk.gIrrep(index));
        for (int srd = sd - 1; srd <= sd + 1; srd += 2) {  // case 2
          const int dru = dim(index + 1, n + 2, su, i), drd = dim(index + 1, n + 2, srd, ird);
          if (dru <= 0 || drd <= 0) continue;
          const double fD = podd(srd + 1) * std::sqrt(3.0 * (srd + 1.0) * (su + 1.0) / (sd + 1.0)) *
                            wigner6j(1, 1, 2, su, srd, sd);
          thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
          parts.assign(1, {fD, need(D.blk(n + 2, su, i, n + 2, srd, ird))});
          if (srd == su)
            parts.push_back({ph(su + 1 - sd) * std::sqrt(0.5 * (su + 1.0) / (sd + 1.0)),
                             need(C.blk(n + 2, su, i, n + 2, srd, ird))});
          const Blk M = tb.combine(parts, dru, drd);
          tb.contract(ob, 1.0, need(T.blk(n, su, i, n + 2, su, i)), false, M, false,
                      need(T.blk(n + 1, sd, id, n + 2, srd, ird)), true);
        }
      }
    }
  }

  // ---------------------------------------------------------------------------------
  // CheMPS2/TensorX.cpp:126-165 (makenewRight / makenewLeft)
  void X_new(const OpT& out) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      tb.declare_output(ob);
      const int n = lay.n_up[ik], s = lay.spin_up[ik], i = lay.irrep_up[ik];
      if (out.moving_right) {
        const double alpha = V(index - 1, index - 1, index - 1, index - 1);
        if (dim(index - 1, n - 2, s, i) > 0 && std::fabs(alpha) > 0.0) {
          const Blk Tb = need(T.blk(n - 2, s, i, n, s, i));
          tb.contract(ob, alpha, Tb, true, Tb, false, kNone, false);
        }
      } else {
        const double alpha = V(index, index, index, index);
        if (dim(index + 1, n + 2, s, i) > 0 && std::fabs(alpha) > 0.0) {
          const Blk Tb = need(T.blk(n, s, i, n + 2, s, i));
          tb.contract(ob, alpha, kNone, false, Tb, false, Tb, true);
        }
      }
    }
  }

  // Symmetrised sandwich: out += W + W^T with W = alpha * opA * M * opC. Emitted as the
  // two contractions W and W^T = alpha * opC^T * M^T * opA^T (same sum as the
  // reference's "mem + mem^T", in a different rounding order).
  void sym_contract(const Blk& ob, double alpha, const Blk& A, bool ta, const Blk& M, bool tm,
                    const Blk& C, bool tc) {
    tb.contract(ob, alpha, A, ta, M, tm, C, tc);
    tb.contract(ob, alpha, C, !tc, M, !tm, A, !ta);
  }

  // CheMPS2/TensorX.cpp:167-371 (addTermQLRight / Left)
  template <class LF>
  void X_QL(const OpT& out, LF Lprev, const OpT& Qprev) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      const int n = lay.n_up[ik], s = lay.spin_up[ik], i = lay.irrep_up[ik];
      for (int geval = 0; geval < 4; geval++) {
        if (out.moving_right) {
          int nu, su2, iu, nd, sd2, idn;
          const int il = irrep_prod(i, bk.gIrrep(index - 1));
          switch (geval) {
            case 0: nu = n - 1; su2 = s - 1; iu = il; nd = n; sd2 = s; idn = i; break;
            case 1: nu = n - 1; su2 = s + 1; iu = il; nd = n; sd2 = s; idn = i; break;
            case 2: nu = n - 2; su2 = s; iu = i; nd = n - 1; sd2 = s - 1; idn = il; break;
            default: nu = n - 2; su2 = s; iu = i; nd = n - 1; sd2 = s + 1; idn = il; break;
          }
          const int du = dim(index - 1, nu, su2, iu), dd = dim(index - 1, nd, sd2, idn);
          if (du <= 0 || dd <= 0) continue;
          const Blk Tu = need(T.blk(nu, su2, iu, n, s, i));
          const Blk Td = need(T.blk(nd, sd2, idn, n, s, i));
          const Blk Qb = need(Qprev.blk(nu, su2, iu, nd, sd2, idn));
          double factor;
          Blk M;
          if (geval < 2) {
            factor = 1.0;
            M = Qb;
          } else {
            factor = ph(s + 1 - sd2) * std::sqrt((sd2 + 1.0) / (s + 1.0));
            thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
            parts.assign(1, {1.0, Qb});
            for (int loca = 0; loca < index - 1; loca++)
              if (bk.gIrrep(index - 1) == bk.gIrrep(loca))
                parts.push_back({V(loca, index - 1, index - 1, index - 1),
                                 need(Lprev(loca).blk(nu, su2, iu, nd, sd2, idn))});
            M = tb.combine(parts, du, dd);
          }
          sym_contract(ob, factor, Tu, true, M, false, Td, false);
        } else {
          int nu, su2, iu, nd, sd2, idn;
          const int irr = irrep_prod(i, bk.gIrrep(index));
          switch (geval) {
            case 0: nu = n; su2 = s; iu = i; nd = n + 1; sd2 = s - 1; idn = irr; break;
            case 1: nu = n; su2 = s; iu = i; nd = n + 1; sd2 = s + 1; idn = irr; break;
            case 2: nu = n + 1; su2 = s - 1; iu = irr; nd = n + 2; sd2 = s; idn = i; break;
            default: nu = n + 1; su2 = s + 1; iu = irr; nd = n + 2; sd2 = s; idn = i; break;
          }
          const int du = dim(index + 1, nu, su2, iu), dd = dim(index + 1, nd, sd2, idn);
          if (du <= 0 || dd <= 0) continue;
          const Blk Tu = need(T.blk(n, s, i, nu, su2, iu));
          const Blk Td = need(T.blk(n, s, i, nd, sd2, idn));
          const Blk Qb = need(Qprev.blk(nu, su2, iu, nd, sd2, idn));
          double factor;
          Blk M;
          if (geval < 2) {
            factor = (sd2 + 1.0) / (s + 1.0);
            M = Qb;
          } else {
            factor = ph(s + 1 - su2) * std::sqrt((su2 + 1.0) / (s + 1.0));
            thread_local std::vector<std::pair<double, Blk>> parts;  // reused: no allocation per block
            parts.assign(1, {1.0, Qb});
            for (int loca = index + 1; loca < L; loca++)
              if (bk.gIrrep(index) == bk.gIrrep(loca))
                parts.push_back({V(index, index, index, loca), need(Lprev(loca).blk(nu, su2, iu, nd, sd2, idn))});
            M = tb.combine(parts, du, dd);
          }
          sym_contract(ob, factor, Tu, false, M, false, Td, true);
        }
      }
    }
  }

  // CheMPS2/TensorX.cpp:373-449 (addTermARight / Left)
  void X_A(const OpT& out, const OpT& A) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      const int n = lay.n_up[ik], s = lay.spin_up[ik], i = lay.irrep_up[ik];
      if (out.moving_right) {
        if (dim(index - 1, n - 2, s, i) <= 0 || dim(index - 1, n, s, i) <= 0) continue;
        sym_contract(ob, std::sqrt(2.0), need(T.blk(n - 2, s, i, n, s, i)), true,
                     need(A.blk(n - 2, s, i, n, s, i)), false, need(T.blk(n, s, i, n, s, i)), false);
      } else {
        if (dim(index + 1, n, s, i) <= 0 || dim(index + 1, n + 2, s, i) <= 0) continue;
        sym_contract(ob, std::sqrt(2.0), need(T.blk(n, s, i, n, s, i)), false,
                     need(A.blk(n, s, i, n + 2, s, i)), false, need(T.blk(n, s, i, n + 2, s, i)), true);
      }
    }
  }

  // CheMPS2/TensorX.cpp:451-535 (addTermCRight / Left)
  void X_C(const OpT& out, const OpT& C) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      const int n = lay.n_up[ik], s = lay.spin_up[ik], i = lay.irrep_up[ik];
      for (int geval = 0; geval < 3; geval++) {
        if (out.moving_right) {
          int nl, sl, il;
          if (geval == 0) { nl = n - 1; sl = s - 1; il = irrep_prod(i, bk.gIrrep(index - 1)); }
          else if (geval == 1) { nl = n - 1; sl = s + 1; il = irrep_prod(i, bk.gIrrep(index - 1)); }
          else { nl = n - 2; sl = s; il = i; }
          if (dim(index - 1, nl, sl, il) <= 0) continue;
          const Blk Tb = need(T.blk(nl, sl, il, n, s, i));
          const double factor = (geval < 2) ? std::sqrt(0.5) : std::sqrt(2.0);
          tb.contract(ob, factor, Tb, true, need(C.blk(nl, sl, il, nl, sl, il)), true, Tb, false);
        } else {
          int nr, sr, irr;
          if (geval == 0) { nr = n + 1; sr = s - 1; irr = irrep_prod(i, bk.gIrrep(index)); }
          else if (geval == 1) { nr = n + 1; sr = s + 1; irr = irrep_prod(i, bk.gIrrep(index)); }
          else { nr = n + 2; sr = s; irr = i; }
          if (dim(index + 1, nr, sr, irr) <= 0) continue;
          const Blk Tb = need(T.blk(n, s, i, nr, sr, irr));
          const double factor = (geval < 2) ? (std::sqrt(0.5) * (sr + 1.0) / (s + 1.0)) : std::sqrt(2.0);
          tb.contract(ob, factor, Tb, false, need(C.blk(nr, sr, irr, nr, sr, irr)), true, Tb, true);
        }
      }
    }
  }

  // CheMPS2/TensorX.cpp:537-645 (addTermDRight / Left)
  void X_D(const OpT& out, const OpT& D) {
    if (!mine(out)) return;
    const OpLayout& lay = *out.lay;
    const int index = lay.index;
    for (int ik = 0; ik < lay.nkappa; ik++) {
      const Blk ob = out.blk_k(ik);
      const int n = lay.n_up[ik], s = lay.spin_up[ik], i = lay.irrep_up[ik];
      for (int geval = 0; geval < 4; geval++) {
        const int a = (geval == 0 || geval == 2) ? s - 1 : s + 1;  // "up"
        const int b = (geval <= 1) ? s - 1 : s + 1;               // "down"
        if (out.moving_right) {
          const int nl = n - 1, il = irrep_prod(i, bk.gIrrep(index - 1));
          if (dim(index - 1, nl, a, il) <= 0 || dim(index - 1, nl, b, il) <= 0) continue;
          const double factor = ph(b + s + 1) * std::sqrt(3.0 * (a + 1)) * wigner6j(1, 1, 2, a, b, s);
          tb.contract(ob, factor, need(T.blk(nl, a, il, n, s, i)), true, need(D.blk(nl, b, il, nl, a, il)), true,
                      need(T.blk(nl, b, il, n, s, i)), false);
        } else {
          const int nr = n + 1, irr = irrep_prod(i, bk.gIrrep(index));
          if (dim(index + 1, nr, a, irr) <= 0 || dim(index + 1, nr, b, irr) <= 0) continue;
          const double factor = ph(s + b + 3) * std::sqrt(3.0 * (a + 1)) * ((b + 1.0) / (s + 1.0)) *
                                wigner6j(1, 1, 2, a, b, s);
          tb.contract(ob, factor, need(T.blk(n, s, i, nr, a, irr)), false, need(D.blk(nr, b, irr, nr, a, irr)), true,
                      need(T.blk(n, s, i, nr, b, irr)), true);
        }
      }
    }
  }
};

}  // namespace

// CheMPS2/DMRGoperators.cpp:243-575 (updateMovingRight) and :576-908 (updateMovingLeft)
void emit_generic_update(TaskBuilder& tb, const SyBookkeeper& bk, const Problem& prob, const MpsT& T, int L,
                         const OpT& out, const OpT& prev) {
  Emit e{tb, bk, prob, T, L};
  e.generic_update(out, prev);
}

void compile_update(TaskBuilder& tb, const UpdateContext& ctx) {
  const SyBookkeeper& bk = *ctx.bk;
  const Problem& prob = *ctx.prob;
  const int L = ctx.L;
  const int index = ctx.index;
  const bool mr = ctx.moving_right;
  BoundaryOps& nx = *ctx.next;
  const BoundaryOps* pv = ctx.prev;
  Emit e{tb, bk, prob, ctx.mps, L};
  std::unordered_map<Ref, int> ids;
  if (ctx.nshards > 1) {
    for (size_t t = 0; t < nx.all.size(); t++) ids[nx.all[t]->base] = static_cast<int>(t);
    // A, B, C and D of one pair receive their complementary sums in stage 2 from the same
    // loop iteration: keep them in one shard.
    for (size_t c2 = 0; c2 < nx.A.size(); c2++)
      for (size_t c3 = 0; c3 < nx.A[c2].size(); c3++) {
        const int id = ids.at(nx.A[c2][c3].base);
        if (c2 > 0) ids[nx.B[c2][c3].base] = id;
        ids[nx.C[c2][c3].base] = id;
        ids[nx.D[c2][c3].base] = id;
      }
    e.shard = ctx.shard;
    e.nshards = ctx.nshards;
    e.tensor_id = &ids;
  }
  const bool edge = mr ? (index == 0) : (index == L - 2);
  auto Lprev = [&](int site) -> const OpT& { return pv->Lop(site); };

  // L tensors
  for (size_t c2 = 0; c2 < nx.L.size(); c2++) {
    if (c2 == 0) e.L_create(nx.L[0]);
    else e.generic_update(nx.L[c2], pv->L[c2 - 1]);
  }
  // F0 / F1 / S0 / S1
  for (size_t c2 = 0; c2 < nx.F0.size(); c2++) {
    for (size_t c3 = 0; c3 < nx.F0[c2].size(); c3++) {
      if (c3 == 0) {
        if (c2 == 0) {
          e.F0_new(nx.F0[c2][0]);
          e.F1_new(nx.F1[c2][0]);
          e.S0_new(nx.S0[c2][0]);
        } else {
          const OpT& Lp = pv->L[c2 - 1];
          e.F0_newL(nx.F0[c2][0], Lp);
          e.F1_newL(nx.F1[c2][0], Lp);
          e.S0_newL(nx.S0[c2][0], Lp);
          e.S1_newL(nx.S1[c2][0], Lp);
        }
      } else {
        e.generic_update(nx.F0[c2][c3], pv->F0[c2][c3 - 1]);
        e.generic_update(nx.F1[c2][c3], pv->F1[c2][c3 - 1]);
        e.generic_update(nx.S0[c2][c3], pv->S0[c2][c3 - 1]);
        if (c2 > 0) e.generic_update(nx.S1[c2][c3], pv->S1[c2][c3 - 1]);
      }
    }
  }
  // A / B / C / D: update part (the cleared tensors at the edge get zero outputs)
  for (size_t c2 = 0; c2 < nx.A.size(); c2++) {
    for (size_t c3 = 0; c3 < nx.A[c2].size(); c3++) {
      if (edge) {
        e.declare_all(nx.A[c2][c3]);
        if (c2 > 0) e.declare_all(nx.B[c2][c3]);
        e.declare_all(nx.C[c2][c3]);
        e.declare_all(nx.D[c2][c3]);
      } else {
        e.generic_update(nx.A[c2][c3], pv->A[c2][c3 + 1]);
        if (c2 > 0) e.generic_update(nx.B[c2][c3], pv->B[c2][c3 + 1]);
        e.generic_update(nx.C[c2][c3], pv->C[c2][c3 + 1]);
        e.generic_update(nx.D[c2][c3], pv->D[c2][c3 + 1]);
      }
    }
  }
  // Q tensors
  const int mps_site = mr ? index : index + 1;
  for (size_t c2 = 0; c2 < nx.Q.size(); c2++) {
    const OpT& q = nx.Q[c2];
    e.declare_all(q);
    if (edge) {
      e.Q_simple(q, mps_site);
    } else {
      e.generic_update(q, pv->Q[c2 + 1]);
      e.Q_simple(q, mps_site);
      e.Q_L(q, Lprev);
      e.Q_AB(q, pv->A[c2 + 1][0], pv->B[c2 + 1][0]);
      e.Q_CD(q, pv->C[c2 + 1][0], pv->D[c2 + 1][0]);
    }
  }
  // X tensor
  e.X_new(nx.X);
  if (!edge) {
    e.generic_update(nx.X, pv->X);
    e.X_QL(nx.X, Lprev, pv->Q[0]);
    e.X_A(nx.X, pv->A[0][0]);
    e.X_C(nx.X, pv->C[0][0]);
    e.X_D(nx.X, pv->D[0][0]);
  }

  // Stage 2: complementary sums with the freshly made pair operators.
  tb.next_stage("update.complementary");
  for (size_t c2 = 0; c2 < nx.A.size(); c2++) {
    for (size_t c3 = 0; c3 < nx.A[c2].size(); c3++) {
      int s1, s2;
      if (mr) { s1 = index + 1 + c3; s2 = index + 1 + c2 + c3; }
      else { s1 = index - c3 - c2; s2 = index - c3; }
      const int iprod = irrep_prod(bk.gIrrep(s1), bk.gIrrep(s2));
      const int nnum = mr ? index + 1 : L - index - 1;
      if (!e.mine(nx.A[c2][c3])) continue;
      for (int num = 0; num < nnum; num++) {
        const OpT& S0n = nx.S0[num][0];
        if (iprod != S0n.irrep()) continue;
        // the two orbitals of the pair operator [num][0] on the swept side
        const int ia = mr ? index - num : index + 1;
        const int ib = mr ? index : index + 1 + num;
        auto hV = [&](int a, int b, int c, int d) { return prob.gMxElement(a, b, c, d); };
        // A and B (absigma part)
        {
          double alpha = mr ? hV(ia, ib, s1, s2) : hV(s1, s2, ia, ib);
          if (c2 == 0 && num == 0) alpha *= 0.5;
          if (c2 > 0 && num > 0) alpha += mr ? hV(ia, ib, s2, s1) : hV(s1, s2, ib, ia);
          for (int ik = 0; ik < nx.A[c2][c3].lay->nkappa; ik++)
            tb.axpy(nx.A[c2][c3].blk_k(ik), alpha, S0n.blk_k(ik), false);
          if (num > 0 && c2 > 0) {
            const double beta = mr ? hV(ia, ib, s1, s2) - hV(ia, ib, s2, s1) : hV(s1, s2, ia, ib) - hV(s1, s2, ib, ia);
            const OpT& S1n = nx.S1[num][0];
            for (int ik = 0; ik < nx.B[c2][c3].lay->nkappa; ik++)
              tb.axpy(nx.B[c2][c3].blk_k(ik), beta, S1n.blk_k(ik), false);
          }
        }
        // C and D (cdf part)
        {
          const OpT& F0n = nx.F0[num][0];
          const OpT& F1n = nx.F1[num][0];
          double ac, ad;
          if (mr) {
            ac = 2 * hV(ia, s1, ib, s2) - hV(ia, s1, s2, ib);
            ad = -hV(ia, s1, s2, ib);
          } else {
            ac = 2 * hV(s1, ia, s2, ib) - hV(s1, ia, ib, s2);
            ad = -hV(s1, ia, ib, s2);
          }
          for (int ik = 0; ik < nx.C[c2][c3].lay->nkappa; ik++)
            tb.axpy(nx.C[c2][c3].blk_k(ik), ac, F0n.blk_k(ik), false);
          for (int ik = 0; ik < nx.D[c2][c3].lay->nkappa; ik++)
            tb.axpy(nx.D[c2][c3].blk_k(ik), ad, F1n.blk_k(ik), false);
          if (num > 0) {
            double tc, td;
            if (mr) {
              tc = 2 * hV(ia, s2, ib, s1) - hV(ia, s2, s1, ib);
              td = -hV(ia, s2, s1, ib);
            } else {
              tc = 2 * hV(s1, ib, s2, ia) - hV(s1, ib, ia, s2);
              td = -hV(s1, ib, ia, s2);
            }
            // CheMPS2/TensorOperator.cpp:418-455 (daxpy_transpose_tensorCD)
            for (const auto& pr : {std::make_pair(&nx.C[c2][c3], std::make_pair(tc, &F0n)),
                                   std::make_pair(&nx.D[c2][c3], std::make_pair(td, &F1n))}) {
              const OpT& dst = *pr.first;
              const double a0 = pr.second.first;
              const OpT& src = *pr.second.second;
              const OpLayout& lay = *dst.lay;
              for (int ik = 0; ik < lay.nkappa; ik++) {
                const int iu = lay.irrep_up[ik], idn = irrep_prod(iu, lay.n_irrep);
                const int su = lay.spin_up[ik], sd = lay.spin_down[ik], nn = lay.n_up[ik];
                double pref = a0;
                if (su != sd)
                  pref *= ph(su - sd) * std::sqrt(mr ? ((su + 1.0) / (sd + 1)) : ((sd + 1.0) / (su + 1)));
                const Blk sb = e.need(src.blk(nn, sd, idn, nn, su, iu));
                tb.axpy(dst.blk_k(ik), pref, sb, true);
              }
            }
          }
        }
      }
    }
  }
}

}  // namespace c2g
