// Minimal stand-in for the reference's inc/solver.h:12-24 (same three virtuals).
#ifndef DROPIN_SOLVER_H
#define DROPIN_SOLVER_H
class Solver {
 public:
  virtual void update(bool input_active) = 0;
  virtual void calculate() = 0;
  virtual void snapshot(TYPE *potential) = 0;
  virtual ~Solver() {}
};
#endif
