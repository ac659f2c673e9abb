// Minimal stand-ins for the reference's element classes (inc/discretization.h): plain
// holders exposing the getters the drop-in adapter reads.  Test infrastructure.
#ifndef DROPIN_DISCRETIZATION_H
#define DROPIN_DISCRETIZATION_H
class discretization {
 public:
  int element, DR, DL, mother;
  bool branching;
  double dX, c_m, r_a, W, K, input_current, rest_pot;
  discretization() : element(0), DR(0), DL(0), mother(0), branching(false), dX(0), c_m(0),
                     r_a(0), W(0), K(0), input_current(0), rest_pot(0) {}
  virtual ~discretization() {}
  int get_element() { return element; }
  int get_DR() { return DR; }
  int get_DL() { return DL; }
  int get_mother() { return mother; }
  bool get_branching() { return branching; }
  double get_dX() { return dX; }
  double get_c_m() { return c_m; }
  double get_r_a() { return r_a; }
  double get_W() { return W; }
  double get_K() { return K; }
  double get_input_current() { return input_current; }
  double get_rest_pot() { return rest_pot; }
};
class Hodgkin_Huxley : public discretization {
 public:
  double m, h, n, g_Na, g_K, G_L, E_Na, E_K, E_L, LS_Na, LS_K;
  double get_m() { return m; }
  double get_h() { return h; }
  double get_n() { return n; }
  double get_g_Na() { return g_Na; }
  double get_g_K() { return g_K; }
  double get_G_L() { return G_L; }
  double get_E_Na() { return E_Na; }
  double get_E_K() { return E_K; }
  double get_E_L() { return E_L; }
  double get_Left_Shift_Na() { return LS_Na; }
  double get_Left_Shift_K() { return LS_K; }
};
#endif
