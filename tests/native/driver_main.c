/* A Formura driver program, written against the generated API only
 * (Formura_Init / Formura_Forward / Formura_Finalize, formura_data,
 * Formura_Navi, to_pos_x), the way the reference's example drivers use it:
 *   - after Formura_Init it writes a deterministic perturbation into
 *     formura_data (the user's init hook);
 *   - it calls Formura_Forward until time_step reaches T_MAX, writing every
 *     value of formura_data (as bit patterns) and the navigator to
 *     data/<time_step>.dat whenever time_step is a multiple of T_OUT;
 *   - halfway it writes into formura_data again (a hook between calls).
 * Built with -DPAIR_HEADER='"X.h"' -DT_MAX=.. -DT_OUT=.. against either the
 * GB300 pair or the oracle pair; the outputs must be byte-identical.
 */
#include <inttypes.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include PAIR_HEADER

#ifndef T_MAX
#define T_MAX 40
#endif
#ifndef T_OUT
#define T_OUT 10
#endif

static uint64_t lcg_state = 0x853c49e6748fea9bull;

static double next_unit(void) {
  lcg_state = lcg_state * 6364136223846793005ull + 1442695040888963407ull;
  return (double)(lcg_state >> 11) * (1.0 / 9007199254740992.0);
}

/* the struct holds Ns fields of equal extent, doubles back to back */
static double* values(size_t* count) {
  *count = sizeof(formura_data) / sizeof(double);
  return (double*)&formura_data;
}

static void perturb(double amplitude) {
  size_t n;
  double* v = values(&n);
  for (size_t i = 0; i < n; ++i) v[i] += amplitude * (next_unit() - 0.5) * (v[i] != 0.0 ? v[i] : 1.0);
}

static void write_snapshot(const Formura_Navi* nv) {
  char fn[256];
  snprintf(fn, sizeof fn, "data/%d.dat", nv->time_step);
  FILE* fp = fopen(fn, "w");
  if (!fp) {
    fprintf(stderr, "cannot open %s\n", fn);
    Formura_Finalize();
    exit(1);
  }
  fprintf(fp, "time_step %d offset_x %d lower_x %d upper_x %d total_grid_x %d\n", nv->time_step,
          nv->offset_x, nv->lower_x, nv->upper_x, nv->total_grid_x);
  for (int i = nv->lower_x; i < nv->upper_x; ++i) fprintf(fp, "x %d %a\n", i, to_pos_x(i, *nv));
  size_t n;
  const double* v = values(&n);
  for (size_t i = 0; i < n; ++i) {
    uint64_t bits;
    memcpy(&bits, &v[i], sizeof bits);
    fprintf(fp, "%016" PRIx64 "\n", bits);
  }
  fclose(fp);
}

int main(int argc, char** argv) {
  Formura_Navi n;
  Formura_Init(&argc, &argv, &n);
  perturb(0.01);
  write_snapshot(&n);
  int touched = 0;
  while (n.time_step < T_MAX) {
    Formura_Forward(&n);
    if (!touched && n.time_step >= T_MAX / 2) {
      perturb(0.001);
      touched = 1;
    }
    if (n.time_step % T_OUT == 0) write_snapshot(&n);
  }
  Formura_Finalize();
  return 0;
}
