// Reference-order auxiliary-field generator (oracle / test infrastructure only).
//
// The reference seeds one global std::mt19937 per MPI rank with seed + rank
// (executables/DQMC.cpp:58).  Every walker is a copy of a prototype DQMCWalker,
// so each walker owns its own std::normal_distribution<double>(0, 1)
// (DQMC/DQMCWalker.h:18, DQMC/DQMCWalker.cpp:20, DQMC/MixedEstimator.cpp:399),
// including that distribution's cached second variate, while all of them draw
// from the rank's single generator.  Live walkers draw nchol normals per step,
// in walker order (DQMC/DQMCWalker.cpp:451-452 and :518-519; dead walkers are
// skipped by DQMC/MixedEstimator.cpp:462).  The comb draws one
// std::uniform_real_distribution<double>(0, 1) value from rank 0's generator
// (DQMC/MixedEstimator.cpp:599-600).
//
// The arithmetic of those distributions is the C++ standard library's; this
// file uses the same library calls, so the oracle replays the reference's
// field sequence exactly.
#include <random>
#include <vector>

struct FieldGen {
  std::mt19937 gen;
  std::vector<std::normal_distribution<double>> normals;
};

extern "C" {

void* fg_create(unsigned seed, int nwalk) {
  FieldGen* g = new FieldGen();
  g->gen = std::mt19937(seed);
  g->normals.assign(nwalk, std::normal_distribution<double>(0., 1.));
  return g;
}

void fg_destroy(void* p) { delete static_cast<FieldGen*>(p); }

// Draw `count` normals for walker `walker` (its own distribution object).
void fg_draw(void* p, int walker, int count, double* out) {
  FieldGen* g = static_cast<FieldGen*>(p);
  for (int i = 0; i < count; i++) out[i] = g->normals[walker](g->gen);
}

// One step of the reference loop: every walker with weight > 1e-8 draws
// `count` normals, in walker order.  Rows of dead walkers are left untouched.
void fg_draw_step(void* p, int nwalk, const double* weights, int count, double* out) {
  FieldGen* g = static_cast<FieldGen*>(p);
  for (int w = 0; w < nwalk; w++) {
    if (weights[w] > 1.e-8)
      for (int i = 0; i < count; i++) out[(size_t)w * count + i] = g->normals[w](g->gen);
  }
}

double fg_uniform(void* p) {
  FieldGen* g = static_cast<FieldGen*>(p);
  std::uniform_real_distribution<double> u(0., 1.);
  return u(g->gen);
}

}  // extern "C"
