#include "twodm.hpp"

#include <cmath>
#include <stdexcept>

#include "symm.hpp"

namespace c2g {

namespace {

// One product P = op(A) B op(C) (A or C may be absent) whose Frobenius product with T_up
// feeds up to three diagram values with their factors.
struct Target {
  int value;
  double factor;
};

// Pass 0 sizes the work, pass 1 records the products, pass 2 the Frobenius products.
struct Sink {
  TaskBuilder* tb = nullptr;
  int pass = 0;
  int64_t woff = 0;
  int vbase = 0;

  void product(const Blk& Tup, const Blk& A, bool ta, const Blk& B, bool tb_, const Blk& C, bool tc,
               std::initializer_list<Target> targets) {
    const int m = Tup.rows, n = Tup.cols;
    if (m <= 0 || n <= 0) return;
    const int64_t K = static_cast<int64_t>(m) * n;
    if (pass == 1) {
      tb->contract(Blk::make(make_ref(kSlotWork, woff), m, n), 1.0, A, ta, B, tb_, C, tc);
    } else if (pass == 2) {
      const Blk up = Blk::make(Tup.ref, 1, static_cast<int>(K), 1);
      const Blk p = Blk::make(make_ref(kSlotWork, woff), static_cast<int>(K), 1, static_cast<int>(K));
      for (const Target& t : targets)
        tb->contract(Blk::make(make_ref(kSlotY, t.value - vbase), 1, 1), t.factor, up, false, p, false, Blk(), false);
    }
    woff += K;
  }
  // factor * < T, T > (no product)
  void self(const Blk& T, int value, double factor) {
    if (pass != 2 || T.rows <= 0 || T.cols <= 0) return;
    const int64_t K = static_cast<int64_t>(T.rows) * T.cols;
    const Blk row = Blk::make(T.ref, 1, static_cast<int>(K), 1);
    const Blk col = Blk::make(T.ref, static_cast<int>(K), 1, static_cast<int>(K));
    tb->contract(Blk::make(make_ref(kSlotY, value - vbase), 1, 1), factor, row, false, col, false, Blk(), false);
  }
};

class Emitter {
 public:
  Emitter(const TwoDMContext& c, Sink& s) : ctx(c), bk(*c.bk), sink(s), i(c.site), nirr(c.bk->getNumberOfIrreps()) {
    Iorb = bk.gIrrep(i);
  }

  void emit(const TwoDMInstance& in) {
    const int v = in.value0;
    switch (in.kind) {
      case kTdmD1: d1(v); break;
      case kTdmD2: d2(v, right().Lop(in.j)); break;
      case kTdmD3to6: {
        const int c1 = in.k - in.j, c2 = in.j - i - 1;
        d3(v, right().S0[c1][c2]);
        d4(v + 1, right().F0[c1][c2]);
        d5(v + 2, right().F0[c1][c2]);
        d6(v + 3, right().F1[c1][c2]);
        break;
      }
      case kTdmD7: d7(v, left().Lop(in.g)); break;
      case kTdmD8to12: {
        const OpT& Ll = left().Lop(in.g);
        const OpT& Lr = right().Lop(in.j);
        const int Ig = bk.gIrrep(in.g);
        d8(v, Ll, Lr, Ig);
        d9to11(v + 1, Ll, Lr, Ig);
        d12(v + 4, Ll, Lr, Ig);
        break;
      }
      case kTdmD13to24: {
        const OpT& Ll = left().Lop(in.g);
        const int Ig = bk.gIrrep(in.g);
        const int c1 = in.k - in.j, c2 = in.j - i - 1;
        d13(v, Ll, right().S0[c1][c2], Ig);
        d14(v + 1, Ll, right().S0[c1][c2], Ig);
        if (in.k > in.j) {
          d15(v + 2, Ll, right().S1[c1][c2], Ig);
          d16(v + 3, Ll, right().S1[c1][c2], Ig);
        }
        for (int first = 1; first >= 0; first--) {  // D17-D20, then D21-D24
          const int o = first ? 4 : 8;
          d17or21(v + o, Ll, right().F0[c1][c2], Ig, first);
          d18or22(v + o + 1, Ll, right().F0[c1][c2], Ig, first);
          d19or23(v + o + 2, Ll, right().F1[c1][c2], Ig, first);
          d20or24(v + o + 3, Ll, right().F1[c1][c2], Ig, first);
        }
        break;
      }
      default: throw std::logic_error("twodm: unknown diagram kind");
    }
  }

 private:
  const TwoDMContext& ctx;
  const CheMPS2::SyBookkeeper& bk;
  Sink& sink;
  const int i, nirr;
  int Iorb = 0;

  const BoundaryOps& left() const {
    if (!ctx.left) throw std::logic_error("twodm: left operators missing");
    return *ctx.left;
  }
  const BoundaryOps& right() const {
    if (!ctx.right) throw std::logic_error("twodm: right operators missing");
    return *ctx.right;
  }
  int dim(int b, int N, int S, int I) const { return (N < 0 || S < 0) ? 0 : bk.gCurrentDim(b, N, S, I); }
  Blk T(int nl, int sl, int il, int nr, int sr, int ir) const { return ctx.T.blk(nl, sl, il, nr, sr, ir); }
  static Blk need(const Blk& b) {
    if (!b.valid) throw std::logic_error("twodm: a block of nonzero dimensions is missing");
    return b;
  }
  template <class F>
  void for_left(F f) const {
    for (int NL = bk.gNmin(i); NL <= bk.gNmax(i); NL++)
      for (int SL = bk.gTwoSmin(i, NL); SL <= bk.gTwoSmax(i, NL); SL += 2)
        for (int IL = 0; IL < nirr; IL++) f(NL, SL, IL);
  }

  // CheMPS2/TwoDM.cpp:642-668
  void d1(int v) {
    for_left([&](int NL, int SL, int IL) {
      if (dim(i, NL, SL, IL) > 0 && dim(i + 1, NL + 2, SL, IL) > 0) sink.self(need(T(NL, SL, IL, NL + 2, SL, IL)), v, SL + 1.0);
    });
  }
  // :670-713
  void d2(int v, const OpT& Lr) {
    for_left([&](int NL, int SL, int IL) {
      for (int SR = SL - 1; SR <= SL + 1; SR += 2) {
        const int IRup = irrep_prod(IL, Iorb);
        if (dim(i, NL, SL, IL) > 0 && dim(i + 1, NL + 1, SR, IRup) > 0 && dim(i + 1, NL + 2, SL, IL) > 0) {
          const double f = phase(SL + 1 - SR) * 0.5 * std::sqrt((SL + 1) * (SR + 1.0));
          sink.product(need(T(NL, SL, IL, NL + 1, SR, IRup)), Blk(), false, need(T(NL, SL, IL, NL + 2, SL, IL)), false,
                       need(Lr.blk(NL + 1, SR, IRup, NL + 2, SL, IL)), true, {{v, f}});
        }
      }
    });
  }
  // :715-753
  void d3(int v, const OpT& S0) {
    for_left([&](int NL, int SL, int IL) {
      if (dim(i, NL, SL, IL) > 0 && dim(i + 1, NL, SL, IL) > 0 && dim(i + 1, NL + 2, SL, IL) > 0)
        sink.product(need(T(NL, SL, IL, NL + 2, SL, IL)), Blk(), false, need(T(NL, SL, IL, NL, SL, IL)), false,
                     need(S0.blk(NL, SL, IL, NL + 2, SL, IL)), false, {{v, std::sqrt(0.5) * (SL + 1)}});
    });
  }
  // :755-791
  void d4(int v, const OpT& F0) {
    for_left([&](int NL, int SL, int IL) {
      if (dim(i, NL, SL, IL) > 0 && dim(i + 1, NL + 2, SL, IL) > 0) {
        const Blk t = need(T(NL, SL, IL, NL + 2, SL, IL));
        sink.product(t, Blk(), false, t, false, need(F0.blk(NL + 2, SL, IL, NL + 2, SL, IL)), false,
                     {{v, std::sqrt(0.5) * (SL + 1)}});
      }
    });
  }
  // :793-832
  void d5(int v, const OpT& F0) {
    for_left([&](int NL, int SL, int IL) {
      for (int SR = SL - 1; SR <= SL + 1; SR += 2) {
        const int IR = irrep_prod(IL, Iorb);
        if (dim(i, NL, SL, IL) > 0 && dim(i + 1, NL + 1, SR, IR) > 0) {
          const Blk t = need(T(NL, SL, IL, NL + 1, SR, IR));
          sink.product(t, Blk(), false, t, false, need(F0.blk(NL + 1, SR, IR, NL + 1, SR, IR)), false,
                       {{v, 0.5 * std::sqrt(0.5) * (SR + 1)}});
        }
      }
    });
  }
  // :834-879
  void d6(int v, const OpT& F1) {
    for_left([&](int NL, int SL, int IL) {
      const int IR = irrep_prod(IL, Iorb);
      for (int SRu = SL - 1; SRu <= SL + 1; SRu += 2)
        for (int SRd = SL - 1; SRd <= SL + 1; SRd += 2) {
          if (!(dim(i, NL, SL, IL) > 0 && dim(i + 1, NL + 1, SRu, IR) > 0 && dim(i + 1, NL + 1, SRd, IR) > 0)) continue;
          const double f = std::sqrt((SRu + 1) / 3.0) * (SRd + 1) * phase(SL + SRd - 1) * wigner6j(1, 1, 2, SRu, SRd, SL);
          sink.product(need(T(NL, SL, IL, NL + 1, SRu, IR)), Blk(), false, need(T(NL, SL, IL, NL + 1, SRd, IR)), false,
                       need(F1.blk(NL + 1, SRd, IR, NL + 1, SRu, IR)), false, {{v, f}});
        }
    });
  }
  // :881-925
  void d7(int v, const OpT& Ll) {
    for_left([&](int NLu, int SLu, int ILu) {
      if (dim(i, NLu, SLu, ILu) <= 0) return;
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2) {
        const int IR = irrep_prod(ILu, Iorb);
        if (!(dim(i, NLu - 1, SLd, IR) > 0 && dim(i + 1, NLu + 1, SLd, IR) > 0)) continue;
        const double f = 0.5 * std::sqrt((SLd + 1) * (SLu + 1.0)) * phase(SLu - SLd + 3);
        sink.product(need(T(NLu, SLu, ILu, NLu + 1, SLd, IR)), need(Ll.blk(NLu - 1, SLd, IR, NLu, SLu, ILu)), true,
                     need(T(NLu - 1, SLd, IR, NLu + 1, SLd, IR)), false, Blk(), false, {{v, f}});
      }
    });
  }
  // :927-979
  void d8(int v, const OpT& Ll, const OpT& Lr, int Ig) {
    for_left([&](int NL, int SLu, int ILu) {
      if (!(dim(i, NL, SLu, ILu) > 0 && dim(i + 1, NL + 2, SLu, ILu) > 0)) return;
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2) {
        const int Id = irrep_prod(ILu, Ig);
        if (!(dim(i, NL - 1, SLd, Id) > 0 && dim(i + 1, NL + 1, SLd, Id) > 0)) continue;
        sink.product(need(T(NL, SLu, ILu, NL + 2, SLu, ILu)), need(Ll.blk(NL - 1, SLd, Id, NL, SLu, ILu)), true,
                     need(T(NL - 1, SLd, Id, NL + 1, SLd, Id)), false, need(Lr.blk(NL + 1, SLd, Id, NL + 2, SLu, ILu)),
                     false, {{v, -0.5 * (SLu + 1)}});
      }
    });
  }
  // :981-1051 (values v: d9, v + 1: d10, v + 2: d11)
  void d9to11(int v, const OpT& Ll, const OpT& Lr, int Ig) {
    for_left([&](int NL, int SLu, int ILu) {
      if (dim(i, NL, SLu, ILu) <= 0) return;
      const int IRu = irrep_prod(ILu, Iorb), ILd = irrep_prod(ILu, Ig), IRd = irrep_prod(ILd, Iorb);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2)
        for (int SRu = SLu - 1; SRu <= SLu + 1; SRu += 2)
          for (int SRd = SRu - 1; SRd <= SRu + 1; SRd += 2) {
            if (!(SLd >= 0 && SRu >= 0 && SRd >= 0 && std::abs(SLd - SRd) <= 1)) continue;
            if (!(dim(i, NL - 1, SLd, ILd) > 0 && dim(i + 1, NL + 1, SRu, IRu) > 0 && dim(i + 1, NL, SRd, IRd) > 0))
              continue;
            const double root = std::sqrt((SRd + 1) * (SLu + 1.0));
            const double f1 = phase(SLu + SRd + 2) * (SRu + 1) * root * wigner6j(SRu, 1, SLu, SLd, 1, SRd);
            const double f2 = 2 * (SRu + 1) * root * wigner6j(SRu, SLd, 2, 1, 1, SLu) * wigner6j(SRu, SLd, 2, 1, 1, SRd);
            const double f3 = (SRd == SLu) ? (SRu + 1) : 0;
            sink.product(need(T(NL, SLu, ILu, NL + 1, SRu, IRu)), need(Ll.blk(NL - 1, SLd, ILd, NL, SLu, ILu)), true,
                         need(T(NL - 1, SLd, ILd, NL, SRd, IRd)), false, need(Lr.blk(NL, SRd, IRd, NL + 1, SRu, IRu)),
                         false, {{v, f1}, {v + 1, f2}, {v + 2, f3}});
          }
    });
  }
  // :1053-1106
  void d12(int v, const OpT& Ll, const OpT& Lr, int Ig) {
    for_left([&](int NL, int SLu, int ILu) {
      if (!(dim(i, NL, SLu, ILu) > 0 && dim(i + 1, NL, SLu, ILu) > 0)) return;
      const int Id = irrep_prod(ILu, Ig);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2) {
        if (!(dim(i, NL - 1, SLd, Id) > 0 && dim(i + 1, NL + 1, SLd, Id) > 0)) continue;
        const double f = phase(SLd + 1 - SLu) * 0.5 * std::sqrt((SLu + 1) * (SLd + 1.0));
        sink.product(need(T(NL, SLu, ILu, NL, SLu, ILu)), need(Ll.blk(NL - 1, SLd, Id, NL, SLu, ILu)), true,
                     need(T(NL - 1, SLd, Id, NL + 1, SLd, Id)), false, need(Lr.blk(NL, SLu, ILu, NL + 1, SLd, Id)),
                     true, {{v, f}});
      }
    });
  }
  // :1108-1162
  void d13(int v, const OpT& Ll, const OpT& S0, int Ig) {
    for_left([&](int NL, int SLu, int ILu) {
      if (!(dim(i, NL, SLu, ILu) > 0 && dim(i + 1, NL + 2, SLu, ILu) > 0)) return;
      const int ILd = irrep_prod(ILu, Ig), IRd = irrep_prod(ILd, Iorb);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2) {
        if (!(dim(i, NL - 1, SLd, ILd) > 0 && dim(i + 1, NL, SLu, IRd) > 0)) continue;
        sink.product(need(T(NL, SLu, ILu, NL + 2, SLu, ILu)), need(Ll.blk(NL - 1, SLd, ILd, NL, SLu, ILu)), true,
                     need(T(NL - 1, SLd, ILd, NL, SLu, IRd)), false, need(S0.blk(NL, SLu, IRd, NL + 2, SLu, ILu)), false,
                     {{v, -0.5 * std::sqrt(0.5) * (SLu + 1)}});
      }
    });
  }
  // :1164-1218
  void d14(int v, const OpT& Ll, const OpT& S0, int Ig) {
    for_left([&](int NL, int SLu, int ILu) {
      if (dim(i, NL, SLu, ILu) <= 0) return;
      const int Id = irrep_prod(ILu, Ig), IRu = irrep_prod(ILu, Iorb);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2) {
        if (!(dim(i, NL - 1, SLd, Id) > 0 && dim(i + 1, NL - 1, SLd, Id) > 0 && dim(i + 1, NL + 1, SLd, IRu) > 0))
          continue;
        const double f = phase(SLd + 1 - SLu) * 0.5 * std::sqrt(0.5 * (SLu + 1) * (SLd + 1));
        sink.product(need(T(NL, SLu, ILu, NL + 1, SLd, IRu)), need(Ll.blk(NL - 1, SLd, Id, NL, SLu, ILu)), true,
                     need(T(NL - 1, SLd, Id, NL - 1, SLd, Id)), false, need(S0.blk(NL - 1, SLd, Id, NL + 1, SLd, IRu)),
                     false, {{v, f}});
      }
    });
  }
  // :1220-1277
  void d15(int v, const OpT& Ll, const OpT& S1, int Ig) {
    for_left([&](int NL, int SLu, int ILu) {
      if (!(dim(i, NL, SLu, ILu) > 0 && dim(i + 1, NL + 2, SLu, ILu) > 0)) return;
      const int ILd = irrep_prod(ILu, Ig), IRd = irrep_prod(ILd, Iorb);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2)
        for (int SRd = SLd - 1; SRd <= SLd + 1; SRd += 2) {
          if (!(dim(i, NL - 1, SLd, ILd) > 0 && dim(i + 1, NL, SRd, IRd) > 0)) continue;
          const double f =
              phase(SLd + SLu + 1) * (SLu + 1) * std::sqrt((SRd + 1) / 3.0) * wigner6j(1, 1, 2, SLu, SRd, SLd);
          sink.product(need(T(NL, SLu, ILu, NL + 2, SLu, ILu)), need(Ll.blk(NL - 1, SLd, ILd, NL, SLu, ILu)), true,
                       need(T(NL - 1, SLd, ILd, NL, SRd, IRd)), false, need(S1.blk(NL, SRd, IRd, NL + 2, SLu, ILu)),
                       false, {{v, f}});
        }
    });
  }
  // :1279-1336
  void d16(int v, const OpT& Ll, const OpT& S1, int Ig) {
    for_left([&](int NL, int SLu, int ILu) {
      if (dim(i, NL, SLu, ILu) <= 0) return;
      const int Id = irrep_prod(ILu, Ig), IRu = irrep_prod(ILu, Iorb);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2)
        for (int SRu = SLu - 1; SRu <= SLu + 1; SRu += 2) {
          if (!(dim(i + 1, NL + 1, SRu, IRu) > 0 && dim(i, NL - 1, SLd, Id) > 0 && dim(i + 1, NL - 1, SLd, Id) > 0))
            continue;
          const double f =
              phase(SRu + SLd + 2) * (SRu + 1) * std::sqrt((SLu + 1) / 3.0) * wigner6j(1, 1, 2, SRu, SLd, SLu);
          sink.product(need(T(NL, SLu, ILu, NL + 1, SRu, IRu)), need(Ll.blk(NL - 1, SLd, Id, NL, SLu, ILu)), true,
                       need(T(NL - 1, SLd, Id, NL - 1, SLd, Id)), false, need(S1.blk(NL - 1, SLd, Id, NL + 1, SRu, IRu)),
                       false, {{v, f}});
        }
    });
  }
  // :1338-1393 (first: D17, otherwise D21 with the F0 block transposed)
  void d17or21(int v, const OpT& Ll, const OpT& F0, int Ig, bool first) {
    for_left([&](int NL, int SLu, int ILu) {
      if (dim(i, NL, SLu, ILu) <= 0) return;
      const int ILd = irrep_prod(ILu, Ig), IRd = irrep_prod(ILd, Iorb);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2) {
        if (!(dim(i + 1, NL, SLu, ILu) > 0 && dim(i, NL - 1, SLd, ILd) > 0 && dim(i + 1, NL, SLu, IRd) > 0)) continue;
        const Blk f0 = first ? F0.blk(NL, SLu, IRd, NL, SLu, ILu) : F0.blk(NL, SLu, ILu, NL, SLu, IRd);
        sink.product(need(T(NL, SLu, ILu, NL, SLu, ILu)), need(Ll.blk(NL - 1, SLd, ILd, NL, SLu, ILu)), true,
                     need(T(NL - 1, SLd, ILd, NL, SLu, IRd)), false, need(f0), !first,
                     {{v, std::sqrt(0.5) * 0.5 * (SLu + 1)}});
      }
    });
  }
  // :1395-1452
  void d18or22(int v, const OpT& Ll, const OpT& F0, int Ig, bool first) {
    for_left([&](int NL, int SLu, int ILu) {
      if (dim(i, NL, SLu, ILu) <= 0) return;
      const int Id = irrep_prod(ILu, Ig), IRu = irrep_prod(ILu, Iorb);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2) {
        if (!(dim(i + 1, NL + 1, SLd, IRu) > 0 && dim(i, NL - 1, SLd, Id) > 0 && dim(i + 1, NL + 1, SLd, Id) > 0))
          continue;
        const Blk f0 = first ? F0.blk(NL + 1, SLd, Id, NL + 1, SLd, IRu) : F0.blk(NL + 1, SLd, IRu, NL + 1, SLd, Id);
        const double f = phase(SLd + 1 - SLu) * 0.5 * std::sqrt(0.5 * (SLu + 1) * (SLd + 1));
        sink.product(need(T(NL, SLu, ILu, NL + 1, SLd, IRu)), need(Ll.blk(NL - 1, SLd, Id, NL, SLu, ILu)), true,
                     need(T(NL - 1, SLd, Id, NL + 1, SLd, Id)), false, need(f0), !first, {{v, f}});
      }
    });
  }
  // :1454-1520
  void d19or23(int v, const OpT& Ll, const OpT& F1, int Ig, bool first) {
    for_left([&](int NL, int SLu, int ILu) {
      if (dim(i, NL, SLu, ILu) <= 0) return;
      const int ILd = irrep_prod(ILu, Ig), IRd = irrep_prod(ILd, Iorb);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2)
        for (int SRd = SLd - 1; SRd <= SLd + 1; SRd += 2) {
          if (!(dim(i + 1, NL, SLu, ILu) > 0 && dim(i, NL - 1, SLd, ILd) > 0 && dim(i + 1, NL, SRd, IRd) > 0)) continue;
          const Blk f1 = first ? F1.blk(NL, SRd, IRd, NL, SLu, ILu) : F1.blk(NL, SLu, ILu, NL, SRd, IRd);
          const double w = wigner6j(1, 1, 2, SLu, SRd, SLd);
          const double f = first ? phase(SLd + SRd - 1) * (SRd + 1) * std::sqrt((SLu + 1) / 3.0) * w
                                 : phase(SLd + SLu - 1) * (SLu + 1) * std::sqrt((SRd + 1) / 3.0) * w;
          sink.product(need(T(NL, SLu, ILu, NL, SLu, ILu)), need(Ll.blk(NL - 1, SLd, ILd, NL, SLu, ILu)), true,
                       need(T(NL - 1, SLd, ILd, NL, SRd, IRd)), false, need(f1), !first, {{v, f}});
        }
    });
  }
  // :1522-1590
  void d20or24(int v, const OpT& Ll, const OpT& F1, int Ig, bool first) {
    for_left([&](int NL, int SLu, int ILu) {
      if (dim(i, NL, SLu, ILu) <= 0) return;
      const int Id = irrep_prod(ILu, Ig), IRu = irrep_prod(ILu, Iorb);
      for (int SLd = SLu - 1; SLd <= SLu + 1; SLd += 2)
        for (int SRu = SLu - 1; SRu <= SLu + 1; SRu += 2) {
          if (!(dim(i + 1, NL + 1, SRu, IRu) > 0 && dim(i, NL - 1, SLd, Id) > 0 && dim(i + 1, NL + 1, SLd, Id) > 0))
            continue;
          const Blk f1 = first ? F1.blk(NL + 1, SLd, Id, NL + 1, SRu, IRu) : F1.blk(NL + 1, SRu, IRu, NL + 1, SLd, Id);
          const double w = wigner6j(1, 1, 2, SRu, SLd, SLu);
          const double f = first ? phase(2 * SLu) * std::sqrt((SLu + 1) * (SRu + 1) * (SLd + 1) / 3.0) * w
                                 : phase(2 * SLu + SRu - SLd) * (SRu + 1) * std::sqrt((SLu + 1) / 3.0) * w;
          sink.product(need(T(NL, SLu, ILu, NL + 1, SRu, IRu)), need(Ll.blk(NL - 1, SLd, Id, NL, SLu, ILu)), true,
                       need(T(NL - 1, SLd, Id, NL + 1, SLd, Id)), false, need(f1), !first, {{v, f}});
        }
    });
  }
};

}  // namespace

int twodm_num_values(int kind) {
  switch (kind) {
    case kTdmD1: return 1;
    case kTdmD2: return 1;
    case kTdmD3to6: return 4;
    case kTdmD7: return 1;
    case kTdmD8to12: return 5;
    case kTdmD13to24: return 12;
    default: throw std::logic_error("twodm: unknown diagram kind");
  }
}

// CheMPS2/TwoDM.cpp:445-628: the loops of FillSite, in order.
std::vector<TwoDMInstance> twodm_instances(const TwoDMContext& ctx) {
  const CheMPS2::SyBookkeeper& bk = *ctx.bk;
  const int L = ctx.L, i = ctx.site;
  std::vector<TwoDMInstance> out;
  int value = 0;
  auto add = [&](int kind, int g, int j, int k) {
    out.push_back(TwoDMInstance{kind, g, j, k, value, 0});
    value += twodm_num_values(kind);
  };
  add(kTdmD1, -1, -1, -1);
  for (int j = i + 1; j < L; j++)
    if (bk.gIrrep(j) == bk.gIrrep(i)) add(kTdmD2, -1, j, -1);
  const int dimTriangle = L - i - 1;
  const int upper = (dimTriangle * (dimTriangle + 1)) / 2;
  int res[2];
  for (int global = 0; global < upper; global++) {
    invert_triangle_two(global, res);
    const int j = L - 1 - res[1], k = j + res[0];
    if (bk.gIrrep(j) == bk.gIrrep(k)) add(kTdmD3to6, -1, j, k);
  }
  for (int g = 0; g < i; g++)
    if (bk.gIrrep(g) == bk.gIrrep(i)) add(kTdmD7, g, -1, -1);
  for (int gj = 0; gj < i * (L - 1 - i); gj++) {
    const int g = gj % i, j = gj / i + i + 1;
    if (bk.gIrrep(g) == bk.gIrrep(j)) add(kTdmD8to12, g, j, -1);
  }
  for (int gjk = 0; gjk < i * upper; gjk++) {
    const int g = gjk % i;
    invert_triangle_two(gjk / i, res);
    const int j = L - 1 - res[1], k = j + res[0];
    if (irrep_prod(bk.gIrrep(g), bk.gIrrep(i)) == irrep_prod(bk.gIrrep(j), bk.gIrrep(k))) add(kTdmD13to24, g, j, k);
  }
  // work sizes
  Sink s;
  s.pass = 0;
  Emitter e(ctx, s);
  for (TwoDMInstance& in : out) {
    s.woff = 0;
    e.emit(in);
    in.work = s.woff;
  }
  return out;
}

void compile_twodm(TaskBuilder& tb, const TwoDMContext& ctx, const std::vector<TwoDMInstance>& inst, size_t first,
                   size_t last) {
  if (first >= last) return;
  Sink s;
  s.tb = &tb;
  s.vbase = inst[first].value0;
  Emitter e(ctx, s);
  s.pass = 1;
  s.woff = 0;
  for (size_t n = first; n < last; n++) e.emit(inst[n]);
  tb.next_stage("twodm.dots");
  s.pass = 2;
  s.woff = 0;
  for (size_t n = first; n < last; n++) e.emit(inst[n]);
  // every value exists as an output, zero when no block contributes
  const int nv = inst[last - 1].value0 + twodm_num_values(inst[last - 1].kind) - s.vbase;
  for (int v = 0; v < nv; v++) tb.declare_output(Blk::make(make_ref(kSlotY, v), 1, 1));
}

void twodm_assemble(CheMPS2::TwoDM& dm, int i, const std::vector<TwoDMInstance>& inst,
                    const std::vector<double>& values) {
  for (const TwoDMInstance& in : inst) {
    const double* d = values.data() + in.value0;
    const int g = in.g, j = in.j, k = in.k;
    switch (in.kind) {
      case kTdmD1:
        dm.set_A(i, i, i, i, 2 * d[0]);
        dm.set_B(i, i, i, i, -2 * d[0]);
        break;
      case kTdmD2:
        dm.set_A(i, j, i, i, 2 * d[0]);
        dm.set_B(i, j, i, i, -2 * d[0]);
        break;
      case kTdmD3to6: {
        const double d3 = d[0], d4 = d[1], d5 = d[2], d6 = d[3];
        dm.set_A(i, i, j, k, 2 * d3);
        dm.set_B(i, i, j, k, -2 * d3);
        dm.set_A(i, j, k, i, -2 * d4 - 2 * d5 - 3 * d6);
        dm.set_B(i, j, k, i, -2 * d4 - 2 * d5 + d6);
        dm.set_A(i, j, i, k, 4 * d4 + 4 * d5);
        dm.set_B(i, j, i, k, 2 * d6);
        break;
      }
      case kTdmD7:
        dm.set_A(g, i, i, i, 2 * d[0]);
        dm.set_B(g, i, i, i, -2 * d[0]);
        break;
      case kTdmD8to12: {
        const double d8 = d[0], d9 = d[1], d10 = d[2], d11 = d[3], d12 = d[4];
        dm.set_A(g, i, j, i, -4 * d8 - d9);
        dm.set_A(g, i, i, j, 2 * d8 + d11);
        dm.set_B(g, i, j, i, d9 - 2 * d10);
        dm.set_B(g, i, i, j, 2 * d8 + 2 * d10 - d11);
        dm.set_A(g, j, i, i, 2 * d12);
        dm.set_B(g, j, i, i, -2 * d12);
        break;
      }
      case kTdmD13to24: {
        const double d13 = d[0], d14 = d[1], d15 = d[2], d16 = d[3];
        dm.set_A(g, i, j, k, 2 * d13 + 2 * d14 + 3 * d15 + 3 * d16);
        dm.set_A(g, i, k, j, 2 * d13 + 2 * d14 - 3 * d15 - 3 * d16);
        dm.set_B(g, i, j, k, -2 * d13 - 2 * d14 + d15 + d16);
        dm.set_B(g, i, k, j, -2 * d13 - 2 * d14 - d15 - d16);
        const double d17 = d[4], d18 = d[5], d19 = d[6], d20 = d[7];
        dm.set_A(g, j, k, i, -2 * d17 - 2 * d18 - 3 * d19 - 3 * d20);
        dm.set_A(g, j, i, k, 4 * d17 + 4 * d18);
        dm.set_B(g, j, k, i, -2 * d17 - 2 * d18 + d19 + d20);
        dm.set_B(g, j, i, k, 2 * d19 + 2 * d20);
        const double d21 = d[8], d22 = d[9], d23 = d[10], d24 = d[11];
        dm.set_A(g, k, j, i, -2 * d21 - 2 * d22 - 3 * d23 - 3 * d24);
        dm.set_A(g, k, i, j, 4 * d21 + 4 * d22);
        dm.set_B(g, k, j, i, -2 * d21 - 2 * d22 + d23 + d24);
        dm.set_B(g, k, i, j, 2 * d23 + 2 * d24);
        break;
      }
      default: throw std::logic_error("twodm: unknown diagram kind");
    }
  }
}

}  // namespace c2g

namespace CheMPS2 {

TwoDM::TwoDM(const Problem* prob, int L) : prob_(prob), L_(L) {
  const size_t n = static_cast<size_t>(L) * L * L * L;
  A_.assign(n, 0.0);
  B_.assign(n, 0.0);
}

// CheMPS2/TwoDM.cpp:76-96
void TwoDM::set_A(int a, int b, int c, int d, double v) {
  A_[at(a, b, c, d)] = v;
  A_[at(b, a, d, c)] = v;
  A_[at(c, d, a, b)] = v;
  A_[at(d, c, b, a)] = v;
}
void TwoDM::set_B(int a, int b, int c, int d, double v) {
  B_[at(a, b, c, d)] = v;
  B_[at(b, a, d, c)] = v;
  B_[at(c, d, a, b)] = v;
  B_[at(d, c, b, a)] = v;
}

void TwoDM::correct_higher_multiplicities() {
  if (prob_->gTwoS() == 0) return;
  const double f = 1.0 / (prob_->gTwoS() + 1.0);
  for (double& x : A_) x *= f;
  for (double& x : B_) x *= f;
}

bool TwoDM::allowed(int a, int b, int c, int d) const {
  return c2g::irrep_prod(prob_->gIrrep(a), prob_->gIrrep(b)) == c2g::irrep_prod(prob_->gIrrep(c), prob_->gIrrep(d));
}

double TwoDM::getTwoDMA_DMRG(int a, int b, int c, int d) const { return allowed(a, b, c, d) ? A_[at(a, b, c, d)] : 0.0; }
double TwoDM::getTwoDMB_DMRG(int a, int b, int c, int d) const { return allowed(a, b, c, d) ? B_[at(a, b, c, d)] : 0.0; }

// CheMPS2/TwoDM.cpp:128-142
double TwoDM::get1RDM_DMRG(int a, int b) const {
  if (prob_->gIrrep(a) != prob_->gIrrep(b)) return 0.0;
  double v = 0.0;
  for (int r = 0; r < L_; r++) v += getTwoDMA_DMRG(a, r, b, r);
  return v / (prob_->gN() - 1.0);
}

// CheMPS2/TwoDM.cpp:144-163
double TwoDM::spin_density_dmrg(int a, int b) const {
  if (prob_->gIrrep(a) != prob_->gIrrep(b)) return 0.0;
  const int two_s = prob_->gTwoS();
  if (two_s <= 0) return 0.0;
  double v = (2 - prob_->gN()) * get1RDM_DMRG(a, b);
  for (int r = 0; r < L_; r++) v -= getTwoDMA_DMRG(a, r, r, b) + getTwoDMB_DMRG(a, r, r, b);
  return 1.5 * v / (0.5 * two_s + 1);
}

int TwoDM::ham2dmrg(int a) const { return prob_->gReorder() ? prob_->gf1(a) : a; }
double TwoDM::getTwoDMA_HAM(int a, int b, int c, int d) const {
  return getTwoDMA_DMRG(ham2dmrg(a), ham2dmrg(b), ham2dmrg(c), ham2dmrg(d));
}
double TwoDM::getTwoDMB_HAM(int a, int b, int c, int d) const {
  return getTwoDMB_DMRG(ham2dmrg(a), ham2dmrg(b), ham2dmrg(c), ham2dmrg(d));
}
double TwoDM::get1RDM_HAM(int a, int b) const { return get1RDM_DMRG(ham2dmrg(a), ham2dmrg(b)); }
double TwoDM::spin_density_ham(int a, int b) const { return spin_density_dmrg(ham2dmrg(a), ham2dmrg(b)); }

// CheMPS2/TwoDM.cpp:205-232
double TwoDM::trace() const {
  double v = 0.0;
  for (int a = 0; a < L_; a++)
    for (int b = 0; b < L_; b++) v += getTwoDMA_DMRG(a, b, a, b);
  return v;
}

double TwoDM::energy() const {
  double v = 0.0;
  for (int a = 0; a < L_; a++)
    for (int b = 0; b < L_; b++)
      for (int c = 0; c < L_; c++)
        for (int d = 0; d < L_; d++) v += getTwoDMA_DMRG(a, b, c, d) * prob_->gMxElement(a, b, c, d);
  return 0.5 * v + prob_->gEconst();
}

}  // namespace CheMPS2
