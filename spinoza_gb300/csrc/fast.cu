// Fast-mode lowering for the fused executor (opt-in, SPZ_EXEC_FAST).
//
// On GB300 every dense FP64 gate is bound by FP64 issue, so fast mode rewrites
// the circuit into mathematically identical ops that need fewer FP64
// instructions (results differ from the exact mode by rounding only):
//
//   * lazy scaling: H, RX and RY are applied as the gate divided by a scalar
//     (1/sqrt2, cos or sin of theta/2, whichever is larger in magnitude, so
//     the remaining coefficient has magnitude <= 1); the scalars multiply into
//     one global factor G.  4 FP64 instructions per pair instead of 8-12.
//   * U(theta, phi, lambda) = P(phi) RY(theta) P(lambda); RZ(theta) =
//     e^{-i theta/2} P(theta); Z = P(pi); Y = i X Z; a diagonal gate with one
//     control (CZ, CP, CRZ) is x_c (b0 + a x_t) in the phase, i.e. three
//     parity terms ({c}, {t}, {c, t}), since x_c x_t = (x_c + x_t - x_c^x_t)/2.
//   * single-qubit phases are not applied where they occur: they are kept as
//     pending terms e^{i alpha parity(x & S)} and pushed through the
//     permutations that follow (X flips alpha and multiplies G by e^{i alpha};
//     CX(c, t) adds c to S when t is in S; SWAP exchanges two bits of S).
//     Before a gate that acts non-diagonally on qubit q, only the q-dependence
//     of the pending terms is applied, as one multiply of the q = 1 half by a
//     small table indexed by the other bits' parities (4 instructions per
//     pair; carried by the lazy op itself when one follows); the rest stays
//     pending.  At the end (or at a measurement) the
//     remaining terms and G are applied in one table multiply.
//
// A brickwork layer of U gates then costs ~8 FP64 instructions per pair and
// gate instead of 14 (7 where the executor fuses two lazy ops over blocks of
// four amplitudes, circuit.cu fuse_lazy_pairs).  Controlled gates other than
// CX stay exact.
#include <cmath>
#include <complex>
#include <vector>

#include "common.cuh"

namespace spz {
namespace {

constexpr double kPiF = 3.14159265358979323846;

struct Term {
  uint64_t S;
  double alpha;
};

struct Lowering {
  uint32_t n;
  std::vector<Term> terms;
  std::complex<double> G{1.0, 0.0};
  int G_exp = 0;  // G is G * 2^G_exp (kept normalised so G never under/overflows)
  std::vector<GateApp>* out;
  std::vector<PhaseTable>* tables;

  void scale(std::complex<double> f) {
    G *= f;
    int e = 0;
    const double mag = std::abs(G);
    if (mag == 0.0) return;
    std::frexp(mag, &e);
    G = std::complex<double>(std::ldexp(G.real(), -e), std::ldexp(G.imag(), -e));
    G_exp += e;
  }

  void add_term(uint64_t S, double alpha) {
    if (S == 0) return;  // e^{i alpha parity(x & 0)} = 1
    for (Term& t : terms)
      if (t.S == S) {
        t.alpha += alpha;
        return;
      }
    terms.push_back(Term{S, alpha});
  }

  void emit(const GateApp& g) { out->push_back(g); }

  void emit_phase(PhaseTable&& tab) {
    GateApp g{};
    g.kind = FK_PHASE;
    g.target = tab.half_bit ? (uint32_t)__builtin_ctzll(tab.half_bit) : 0;
    g.target2 = g.target;
    g.table = (int32_t)tables->size();
    g.touch = tab.half_bit;
    for (int j = 0; j < tab.m; ++j) g.touch |= tab.mask[j];
    tables->push_back(std::move(tab));
    out->push_back(g);
  }

  // The q-dependence of the pending terms, as tables for the q = 1 half (at
  // most kPhaseMaxTerms terms each); the q-independent rest stays pending.
  std::vector<PhaseTable> take_half(int q) {
    const uint64_t qb = 1ull << q;
    std::vector<Term> hit, keep;
    for (const Term& t : terms) ((t.S & qb) ? hit : keep).push_back(t);
    terms.swap(keep);
    std::vector<PhaseTable> out;
    for (size_t b = 0; b < hit.size(); b += kPhaseMaxTerms) {
      PhaseTable tab;
      tab.half_bit = qb;
      tab.m = (int)std::min<size_t>(kPhaseMaxTerms, hit.size() - b);
      for (int j = 0; j < tab.m; ++j) tab.mask[j] = hit[b + j].S & ~qb;
      const size_t E = 1ull << tab.m;
      tab.re.resize(E);
      tab.im.resize(E);
      for (size_t idx = 0; idx < E; ++idx) {
        double ang = 0.0;
        for (int j = 0; j < tab.m; ++j) {  // x_q = 1: e^{i a (1 - 2 p')}
          const double a = hit[b + j].alpha;
          ang += ((idx >> j) & 1) ? -a : a;
        }
        tab.re[idx] = std::cos(ang);
        tab.im[idx] = std::sin(ang);
      }
      out.push_back(std::move(tab));
    }
    for (const Term& t : hit) add_term(t.S & ~qb, t.alpha);  // e^{i a p'} stays pending
    return out;
  }

  // Apply the q-dependence of the pending terms to the q = 1 half.
  void flush_half(int q) {
    for (PhaseTable& tab : take_half(q)) emit_phase(std::move(tab));
  }

  // A lazy op on q preceded by the q-dependence of the pending terms: the last
  // (or only) table rides on the lazy op itself (the op multiplies s1 by its
  // entry before the rotation), the others are separate phase ops.
  void emit_lazy(int kind, int q, double coef) {
    std::vector<PhaseTable> tabs = take_half(q);
    GateApp g = make(kind, (uint32_t)q, coef);
    if (!tabs.empty()) {
      for (size_t j = 0; j + 1 < tabs.size(); ++j) emit_phase(std::move(tabs[j]));
      PhaseTable& last = tabs.back();
      g.table = (int32_t)tables->size();
      g.touch = last.half_bit;
      for (int j = 0; j < last.m; ++j) g.touch |= last.mask[j];
      tables->push_back(std::move(last));
    }
    emit(g);
  }

  // Apply every pending term and the global factor.
  void flush_all() {
    const std::complex<double> g = std::ldexp(1.0, G_exp) * G;
    const bool unit = std::abs(g - std::complex<double>(1.0, 0.0)) == 0.0;
    if (terms.empty() && unit) return;
    size_t b = 0;
    do {
      PhaseTable tab;
      tab.m = (int)std::min<size_t>(kPhaseMaxTerms, terms.size() - b);
      for (int j = 0; j < tab.m; ++j) tab.mask[j] = terms[b + j].S;
      const bool last = b + tab.m >= terms.size();
      const size_t E = 1ull << tab.m;
      tab.re.resize(E);
      tab.im.resize(E);
      for (size_t idx = 0; idx < E; ++idx) {
        double ang = 0.0;
        for (int j = 0; j < tab.m; ++j)
          if ((idx >> j) & 1) ang += terms[b + j].alpha;
        std::complex<double> v = std::polar(1.0, ang);
        if (last) v *= g;
        tab.re[idx] = v.real();
        tab.im[idx] = v.imag();
      }
      emit_phase(std::move(tab));
      b += tab.m;
    } while (b < terms.size());
    terms.clear();
    G = 1.0;
    G_exp = 0;
  }

  // Keep G within range: fold it into the amplitudes when it drifts far.
  void renormalise() {
    if (G_exp > -400 && G_exp < 400) return;
    PhaseTable tab;
    tab.m = 0;
    const std::complex<double> g = std::ldexp(1.0, G_exp) * G;
    tab.re = {g.real()};
    tab.im = {g.imag()};
    emit_phase(std::move(tab));
    G = 1.0;
    G_exp = 0;
  }

  void push_x(int t) {
    const uint64_t tb = 1ull << t;
    for (Term& term : terms)
      if (term.S & tb) {
        scale(std::polar(1.0, term.alpha));
        term.alpha = -term.alpha;
      }
  }

  void push_cx(int c, int t) {
    const uint64_t tb = 1ull << t, cb = 1ull << c;
    for (Term& term : terms)
      if (term.S & tb) term.S ^= cb;
    merge();
  }

  void push_swap(int a, int b) {
    const uint64_t ab = 1ull << a, bb = 1ull << b;
    for (Term& term : terms) {
      const bool ba = (term.S & ab) != 0, bbit = (term.S & bb) != 0;
      if (ba != bbit) term.S ^= ab | bb;
    }
    merge();
  }

  void merge() {  // combine terms with equal masks; masks that became empty are constants
    std::vector<Term> old;
    old.swap(terms);
    for (const Term& t : old) add_term(t.S, t.alpha);
  }

  GateApp make(int kind, uint32_t target, double coef) {
    GateApp g{};
    g.kind = kind;
    g.target = target;
    g.target2 = target;
    g.c.cs = coef;
    return g;
  }

  // RX / RY with cos and sin of theta/2, after the q-dependence of the
  // pending phases.
  void lazy_rotation(bool is_x, int q, double c, double s) {
    if (std::fabs(c) >= std::fabs(s)) {
      emit_lazy(is_x ? FK_LAZY_RX_A : FK_LAZY_RY_A, q, s / c);
      scale(c);
    } else {
      emit_lazy(is_x ? FK_LAZY_RX_B : FK_LAZY_RY_B, q, c / s);
      scale(s);
    }
    renormalise();
  }

  void gate(const GateApp& g) {
    const uint64_t controls = g.ones | g.zeros;
    const int q = (int)g.target;
    if (g.cond >= 0) {  // applied or not by a device-side outcome: stays exact
      if (!is_diagonal(g.kind)) {  // a diagonal gate commutes with the pending phases
        flush_half(q);
        if (g.kind == SPZ_GATE_SWAP) flush_half((int)g.target2);
      }
      emit(g);
      return;
    }
    if (is_diagonal(g.kind)) {
      if (controls == 0) {
        switch (g.kind) {
          case SPZ_GATE_Z: add_term(1ull << q, kPiF); return;
          case SPZ_GATE_P: add_term(1ull << q, std::atan2(g.c.sn, g.c.cs)); return;
          default: {  // RZ = e^{-i theta/2} P(theta): d1/d0 = e^{i theta}
            const std::complex<double> d0(g.c.d0re, g.c.d0im), d1(g.c.d1re, g.c.d1im);
            add_term(1ull << q, std::arg(d1 / d0));
            scale(d0);
            return;
          }
        }
      }
      if (g.zeros == 0 && __builtin_popcountll(g.ones) == 1) {
        // One control c: the phase is x_c (b0 + a x_t), and
        // x_c x_t = (x_c + x_t - (x_c xor x_t)) / 2, so three parity terms.
        const int cq = __builtin_ctzll(g.ones);
        double b0 = 0.0, a;
        switch (g.kind) {
          case SPZ_GATE_Z: a = kPiF; break;
          case SPZ_GATE_P: a = std::atan2(g.c.sn, g.c.cs); break;
          default: {  // RZ: d0 on x_t = 0, d1 on x_t = 1 (both of modulus 1)
            const std::complex<double> d0(g.c.d0re, g.c.d0im), d1(g.c.d1re, g.c.d1im);
            b0 = std::arg(d0);
            a = std::arg(d1 / d0);
          }
        }
        add_term(1ull << cq, b0 + 0.5 * a);
        add_term(1ull << q, 0.5 * a);
        add_term((1ull << cq) | (1ull << q), -0.5 * a);
        return;
      }
      emit(g);  // other controlled diagonals: they commute with the pending terms
      return;
    }
    if (controls == 0) {
      switch (g.kind) {
        case SPZ_GATE_X: push_x(q); emit(g); return;
        case SPZ_GATE_Y:  // Y = i X Z
          add_term(1ull << q, kPiF);
          push_x(q);
          emit(make(SPZ_GATE_X, q, 0.0));
          scale(std::complex<double>(0.0, 1.0));
          return;
        case SPZ_GATE_SWAP: push_swap((int)g.target, (int)g.target2); emit(g); return;
        case SPZ_GATE_H:
          emit_lazy(FK_LAZY_H, q, 0.0);
          scale(std::sqrt(0.5));
          renormalise();
          return;
        case SPZ_GATE_RX:  // cs = cos(theta/2), sn = sin(theta/2)
        case SPZ_GATE_RY:
          lazy_rotation(g.kind == SPZ_GATE_RX, q, g.c.cs, g.c.sn);
          return;
        case SPZ_GATE_U: {
          // U = [[ct, -e^{i l} st], [e^{i p} st, e^{i(p+l)} ct]] = P(p) RY P(l), with
          // g = [(a,0), (k,l), (q,r), (s,t)].  RY's cos is ct = a and its sin is
          // |g10|; lambda = arg(-g01), phi = arg(g10) (for st = 0 the phase sits
          // in g11 / ct and lambda = 0).
          const double ct = g.c.a, st = std::hypot(g.c.q, g.c.r);
          double lambda = 0.0, phi;
          if (st > 0.0) {
            lambda = std::atan2(-g.c.l, -g.c.k);
            phi = std::atan2(g.c.r, g.c.q);
          } else {
            phi = ct < 0.0 ? std::atan2(-g.c.t, -g.c.s) : std::atan2(g.c.t, g.c.s);
          }
          add_term(1ull << q, lambda);
          lazy_rotation(false, q, ct, st);
          add_term(1ull << q, phi);
          return;
        }
        default: break;
      }
    }
    if (g.kind == SPZ_GATE_X && g.zeros == 0 && __builtin_popcountll(g.ones) == 1) {
      push_cx(__builtin_ctzll(g.ones), q);
      emit(g);
      return;
    }
    // Any other gate stays exact; its non-diagonal qubits must first carry no
    // pending phase dependence.
    flush_half(q);
    if (g.kind == SPZ_GATE_SWAP) flush_half((int)g.target2);
    emit(g);
  }
};

}  // namespace

void lower_fast(const std::vector<GateApp>& in, uint32_t n, std::vector<GateApp>* out,
                std::vector<PhaseTable>* tables) {
  Lowering L;
  L.n = n;
  L.out = out;
  L.tables = tables;
  for (const GateApp& g : in) L.gate(g);
  L.flush_all();
}

}  // namespace spz
