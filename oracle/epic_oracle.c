/* ORACLE TEST INFRASTRUCTURE — not part of the product.
 *
 * Plain-C restatement of the reference's time-step loop; see epic_oracle.h.
 * Each function names the reference lines it follows.  Expressions keep the
 * reference's association order so results match it bit for bit when built
 * with -ffp-contract=off (oracle/build_oracle.py).
 */
#include "epic_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define IDX(i, j) ((long)(i) * ny + (j))

/* ------------------------------------------------------------------ RNG --- */
/* MT19937 (Matsumoto & Nishimura 1998) with the default seeding of
 * std::mt19937, and std::generate_canonical<double, 53>: two 32-bit outputs
 * a, b give (a + b * 2^32) / 2^64, clamped below 1.  The reference's Rnd
 * (include/domain.h:218-231) is mt19937 seeded with 0 feeding
 * uniform_real_distribution<double>(0, 1). */
void or_rng_seed(or_rng* r, uint32_t seed) {
  r->mt[0] = seed;
  for (int i = 1; i < 624; i++) r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
  r->mti = 624;
}

uint32_t or_rng_u32(or_rng* r) {
  if (r->mti >= 624) {
    for (int i = 0; i < 624; i++) {
      uint32_t y = (r->mt[i] & 0x80000000u) | (r->mt[(i + 1) % 624] & 0x7fffffffu);
      r->mt[i] = r->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    r->mti = 0;
  }
  uint32_t y = r->mt[r->mti++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

double or_rng_uniform(or_rng* r) {
  double sum = 0.0, tmp = 1.0;
  sum += (double)or_rng_u32(r) * tmp;
  tmp *= 4294967296.0;
  sum += (double)or_rng_u32(r) * tmp;
  tmp *= 4294967296.0;
  double ret = sum / tmp;
  if (ret >= 1.0) ret = nextafter(1.0, 0.0);
  return ret;
}

/* ----------------------------------------------------------- loading --- */
/* Init::SampleVel, src/init.cpp:104-107: v_th * sqrt(2) * (u1 + u2 + u3 - 1.5).
 * The reference leaves the order of the three draws to the compiler; GCC
 * evaluates them left to right (pinned against oracle/_ref). */
double or_sample_vel(or_rng* r, double mass, double temp) {
  double v_th = sqrt(2 * OR_K_B * temp * (OR_QE / OR_K_B) / mass);
  double u1 = or_rng_uniform(r);
  double u2 = or_rng_uniform(r);
  double u3 = or_rng_uniform(r);
  return v_th * sqrt(2) * (u1 + u2 + u3 - 1.5);
}

/* ------------------------------------------------------- conductors --- */
/* Grid::IsGrid over the grids (src/grid.cpp:11-65, src/electrode.cpp:20-26):
 * grids are OR_GRID_WORDS doubles each, {0, min_x, max_x, min_y, max_y, -, -, V}
 * (ReactConductorGrid) or {1, x_center, y_center, electrodes, grid_radius,
 * electrode_radius, -, V} (CircularGrid).  A circular grid has electrodes only
 * once CircularGrid::initialize has run (inside gssolver), so circles_live = 0
 * leaves it out. */
static void electrode_center(const double* g, int k, double* ex, double* ey) {
  const int num = (int)g[3];
  const double theta = k * (2.0 * OR_M_PI / num);  /* src/grid.cpp:52-56 */
  *ex = (int)g[1] + g[4] * cos(theta);
  *ey = (int)g[2] + g[4] * sin(theta);
}

int or_in_conductors(const double* grids, int ng, int circles_live, double x, double y) {
  for (int k = 0; k < ng; k++) {
    const double* g = grids + OR_GRID_WORDS * k;
    if (g[0] == 0) {
      if (x >= (int)g[1] && x <= (int)g[2] && y >= (int)g[3] && y <= (int)g[4]) return 1;
    } else if (circles_live) {
      for (int e = 0; e < (int)g[3]; e++) {
        double ex, ey;
        electrode_center(g, e, &ex, &ey);
        double dx = x - ex, dy = y - ey;
        double distance_squared = dx * dx + dy * dy;
        double radius_squared = g[5] * g[5];
        if (distance_squared <= radius_squared) return 1;
      }
    }
  }
  return 0;
}

/* Grid::initialize of every grid, in order, as gssolver runs it before its
 * iterations (src/field.cpp:100-103): ReactConductorGrid sets rho on the border
 * of its node rectangle (src/grid.cpp:67-85), each electrode of a circular grid
 * sets rho at 100 points of its circle (src/electrode.cpp:4-17).  Nodes outside
 * the grid are skipped (the reference's rectangle loop does not check). */
void or_conductor_rho(const or_domain* d, const double* grids, int ng, double* rho) {
  const int nx = d->nx, ny = d->ny;
  for (int k = 0; k < ng; k++) {
    const double* g = grids + OR_GRID_WORDS * k;
    if (g[0] == 0) {
      int min_i = (int)((((int)g[1]) - d->x0) / d->dx), max_i = (int)((((int)g[2]) - d->x0) / d->dx);
      int min_j = (int)((((int)g[3]) - d->y0) / d->dy), max_j = (int)((((int)g[4]) - d->y0) / d->dy);
      for (int i = min_i; i <= max_i; i++)
        for (int j = min_j; j <= max_j; j++)
          if ((i == min_i || i == max_i || j == min_j || j == max_j) && i >= 0 && i < nx && j >= 0 && j < ny)
            rho[IDX(i, j)] = g[7];
    } else {
      for (int e = 0; e < (int)g[3]; e++) {
        double ex, ey;
        electrode_center(g, e, &ex, &ey);
        const int N = 100;
        for (int q = 0; q < N; q++) {
          double theta = 2.0 * q * OR_M_PI / N;
          int x = (int)(ex + g[5] * cos(theta) + 0.5);
          int y = (int)(ey + g[5] * sin(theta) + 0.5);
          if (x >= 0 && x < nx && y >= 0 && y < ny) rho[IDX(x, y)] = g[7];
        }
      }
    }
  }
}

/* src/init.cpp:22-92, with the rejection of positions inside a conductor
 * (:71-86): a rejected "random" position is drawn again; the other load types
 * repeat the same position, where the reference loops forever (returns -2). */
int or_load_c(const or_domain* d, or_rng* r, const char* type, int n_arg, double mass, double temp, double vsx,
              double vsy, long n, double* out, const double* grids, int ng);
int or_load(const or_domain* d, or_rng* r, const char* type, int n_arg, double mass, double temp, double vsx,
            double vsy, long n, double* out) {
  return or_load_c(d, r, type, n_arg, mass, temp, vsx, vsy, n, out, 0, 0);
}

int or_load_c(const or_domain* d, or_rng* r, const char* type, int n_arg, double mass, double temp, double vsx,
              double vsy, long n, double* out, const double* grids, int ng) {
  int kind;
  if (strcmp(type, "random") == 0) kind = 0;
  else if (strcmp(type, "uniform") == 0) kind = 1;
  else if (strcmp(type, "sin") == 0) kind = 2;
  else if (strcmp(type, "cos") == 0) kind = 3;
  else return -1;
  for (long p = 0; p < n; p++) {
    double x = 0, y = 0;
    for (;;) {
    if (kind == 0) {
      x = d->x0 + d->Lx * or_rng_uniform(r);
      y = d->y0 + d->Ly * or_rng_uniform(r);
    } else if (kind == 1) {
      int nxp = (int)sqrt((double)n);
      int px = (int)(p % nxp), py = (int)(p / nxp);
      x = d->x0 + px * (d->Lx / (nxp - 1));
      y = d->y0 + py * (d->Ly / (nxp - 1));
    } else {
      x = d->x0 + p * (d->Lx / (n - 1));
      y = d->y0 + p * (d->Ly / (n - 1));
      double kx = 2 * OR_PI * n_arg / d->Lx;
      double ky = 2 * OR_PI * n_arg / d->Ly;
      if (kind == 2) {
        x += sin(kx * x);
        y += sin(ky * y);
      } else {
        x += cos(kx * x);
        y += cos(ky * y);
      }
    }
    if (!or_in_conductors(grids, ng, 0, x, y)) break;
    if (kind != 0) return -2;
    }
    double vx = or_sample_vel(r, mass, temp) + vsx * d->vel_norm;
    double vy = or_sample_vel(r, mass, temp) + vsy * d->vel_norm;
    /* The reference loads vz = 0 (src/init.cpp:88, with SampleVel commented
     * out there); the 3V extension draws it like vx and vy, after them. */
    double vz = d->load_3v ? or_sample_vel(r, mass, temp) : 0;
    vx /= d->vel_norm;
    vy /= d->vel_norm;
    vz /= d->vel_norm;
    double* q = out + 5 * p;
    q[0] = x; q[1] = y; q[2] = vx; q[3] = vy; q[4] = vz;
  }
  return 0;
}

/* --------------------------------------------------------- emitters --- */
/* Emitter::inject (src/emitter.cpp:5-36) of one emitter em = {x0, y0, x1, y1,
 * temp, numparticle, vdx, vdy, species_idx1, species_idx2}.  The reference
 * draws positions from a generator seeded by std::random_device
 * (Domain::unirand, src/domain.cpp:288-299), so they come in as pos_u (two
 * uniforms per point, used as std::uniform_real_distribution does:
 * u (b - a) + a); velocities are Init::SampleVel (src/init.cpp:110-114) on the
 * global stream r, or on vel_u when given (6 uniforms per particle, stride 12
 * per point).  Appends to out1 (and out2 when the indices differ); returns -1
 * when a species runs out of capacity. */
static double sample_vel_t(or_rng* r, const double** vu, double mass, double temp) {
  double v_th = sqrt(2 * OR_K_B * temp * (OR_QE / OR_K_B) / mass);
  double u1, u2, u3;
  if (*vu) {
    u1 = (*vu)[0]; u2 = (*vu)[1]; u3 = (*vu)[2];
    *vu += 3;
  } else {
    u1 = or_rng_uniform(r); u2 = or_rng_uniform(r); u3 = or_rng_uniform(r);
  }
  return v_th * sqrt(2) * (u1 + u2 + u3 - 1.5);
}

int or_inject(const or_domain* d, const double* em, double mass1, double mass2, or_rng* r, const double* pos_u,
              const double* vel_u, double* out1, long* n1, long cap1, double* out2, long* n2, long cap2) {
  const int num = (int)em[5];
  const int two = (int)em[8] != (int)em[9];
  for (int p = 0; p < num; p++) {
    double x = pos_u[2 * p] * (em[2] - em[0]) + em[0];
    double y = pos_u[2 * p + 1] * (em[3] - em[1]) + em[1];
    const double* vu = vel_u ? vel_u + 12 * (long)p : 0;
    double vx1 = sample_vel_t(r, &vu, mass1, em[4]) + em[6] * d->vel_norm;
    double vy1 = sample_vel_t(r, &vu, mass1, em[4]) + em[7] * d->vel_norm;
    double vz1 = 0.0;
    vx1 /= d->vel_norm;
    vy1 /= d->vel_norm;
    vz1 /= d->vel_norm;
    if (*n1 >= cap1) return -1;
    double* q = out1 + 5 * (*n1)++;
    q[0] = x; q[1] = y; q[2] = vx1; q[3] = vy1; q[4] = vz1;
    if (two) {
      double vx2 = sample_vel_t(r, &vu, mass2, em[4]) + em[6] * d->vel_norm;
      double vy2 = sample_vel_t(r, &vu, mass2, em[4]) + em[7] * d->vel_norm;
      double vz2 = 0.0;
      vx2 /= d->vel_norm;
      vy2 /= d->vel_norm;
      vz2 /= d->vel_norm;
      if (*n2 >= cap2) return -1;
      q = out2 + 5 * (*n2)++;
      q[0] = x; q[1] = y; q[2] = vx2; q[3] = vy2; q[4] = vz2;
    }
  }
  return 0;
}

/* ----------------------------------------------------------- deposit --- */
/* Species::ScatterSpecies_serial (src/species.cpp:172-226) with
 * Domain::Scatter (src/domain.cpp:205-228) and XtoL/YtoL (:257-264). */
long or_scatter(const or_domain* d, const double* part, long n, double spwt, double* den) {
  const int nx = d->nx, ny = d->ny;
  long bad = 0;
  memset(den, 0, sizeof(double) * (size_t)nx * ny);
  for (long p = 0; p < n; p++) {
    double lx = (part[5 * p] - d->x0) / d->dx;
    double ly = (part[5 * p + 1] - d->y0) / d->dy;
    int i = (int)lx, j = (int)ly;
    double di = lx - i, dj = ly - j;
    if (d->shape == OR_NGP) {
      int gx = (int)round(lx), gy = (int)round(ly);
      if (gx < 0 || gx >= nx || gy < 0 || gy >= ny) { bad++; continue; }
      den[IDX(gx, gy)] += spwt;
    } else {
      if (i < 0 || i + 1 >= nx || j < 0 || j + 1 >= ny) { bad++; continue; }
      den[IDX(i, j)] += spwt * (1 - di) * (1 - dj);
      den[IDX(i + 1, j)] += spwt * (di) * (1 - dj);
      den[IDX(i, j + 1)] += spwt * (1 - di) * (dj);
      den[IDX(i + 1, j + 1)] += spwt * (di) * (dj);
    }
  }
  double cell_area = d->dx * d->dy;
  double L2 = d->L * d->L;
  double div = cell_area * L2 * d->density;
  for (long k = 0; k < (long)nx * ny; k++) den[k] /= div;
  if (d->bc == OR_PBC) {
    for (int i = 0; i < nx; i++) {
      den[IDX(i, 0)] += den[IDX(i, ny - 1)];
      den[IDX(i, ny - 1)] = den[IDX(i, 0)];
    }
    for (int j = 0; j < ny; j++) {
      den[IDX(0, j)] += den[IDX(nx - 1, j)];
      den[IDX(nx - 1, j)] = den[IDX(0, j)];
    }
  } else {
    den[IDX(0, 0)] *= 0.25;
    den[IDX(0, ny - 1)] *= 0.25;
    den[IDX(nx - 1, 0)] *= 0.25;
    den[IDX(nx - 1, ny - 1)] *= 0.25;
    for (int i = 1; i < nx - 1; i++) {
      den[IDX(i, 0)] *= 0.5;
      den[IDX(i, ny - 1)] *= 0.5;
    }
    for (int j = 1; j < ny - 1; j++) {
      den[IDX(0, j)] *= 0.5;
      den[IDX(nx - 1, j)] *= 0.5;
    }
  }
  return bad;
}

/* Domain::ComputeRho (src/domain.cpp:194-202): rho = sum_s den_s * (q_s/e). */
void or_compute_rho(const or_domain* d, int nsp, const double* const* dens, const double* charges, double* rho) {
  long nn = (long)d->nx * d->ny;
  for (long k = 0; k < nn; k++) rho[k] = 0;
  for (int s = 0; s < nsp; s++) {
    double c = charges[s] * (1 / OR_QE);
    for (long k = 0; k < nn; k++) {
      double t = dens[s][k] * c;
      rho[k] = rho[k] + t;
    }
  }
}

static double dot(const double* a, const double* b, long n);

/* ------------------------------------------------ Poisson extensions --- */
/* Extensions with no reference counterpart (restatements of this project's
 * own definitions; the tests pin them against direct solves).  The reference
 * solves with phi = 0 on all four edges; these put the Poisson problem on
 *   periodic:     unknowns i in [0, nx-2], j in [0, ny-2], both directions
 *                 periodic (node nx-1 is node 0, node ny-1 is node 0); the
 *                 right-hand side is projected onto zero mean and phi is
 *                 returned with zero mean over the unknowns;
 *   dirichlet_x:  unknowns i in [1, nx-2], j in [0, ny-2]; phi = 0 on the
 *                 x walls i = 0 and i = nx-1, periodic in y.
 * The lattice of unknowns has R rows (x index i = row + i0) of C = ny - 1
 * columns (y index j = col), index q = row * C + col. */

/* Correctly rounded sum: a long accumulator of 32-bit digits, digit k worth
 * 2^(32k - 1100), so every finite double is at most three shifted digits and
 * the total is exact until the single rounding at the end. */
#define OR_ACC_DIGITS 72
double or_exact_sum(const double* x, long n) {
  int64_t acc[OR_ACC_DIGITS];
  memset(acc, 0, sizeof(acc));
  for (long t = 0; t < n; t++) {
    uint64_t b;
    memcpy(&b, &x[t], 8);
    int e = (int)((b >> 52) & 0x7FF);
    uint64_t m = b & 0xFFFFFFFFFFFFFull;
    if (e == 0x7FF) return NAN;
    if (e) m |= 1ull << 52;
    else e = 1;
    if (!m) continue;
    const int p = e + 25; /* m * 2^(e - 1075) = m * 2^(p - 1100) */
    const int k = p / 32, sft = p % 32;
    const unsigned __int128 v = (unsigned __int128)m << sft;
    const int64_t d0 = (int64_t)(uint32_t)v, d1 = (int64_t)(uint32_t)(v >> 32), d2 = (int64_t)(uint32_t)(v >> 64);
    if (b >> 63) {
      acc[k] -= d0; acc[k + 1] -= d1; acc[k + 2] -= d2;
    } else {
      acc[k] += d0; acc[k + 1] += d1; acc[k + 2] += d2;
    }
  }
  /* digits to [0, 2^32) with the carries moved up; the top digit keeps the sign */
  for (int k = 0; k < OR_ACC_DIGITS - 1; k++) {
    const int64_t c = acc[k] >> 32;
    acc[k] -= c * ((int64_t)1 << 32);
    acc[k + 1] += c;
  }
  const int neg = acc[OR_ACC_DIGITS - 1] < 0;
  if (neg) {
    for (int k = 0; k < OR_ACC_DIGITS; k++) acc[k] = -acc[k];
    for (int k = 0; k < OR_ACC_DIGITS - 1; k++) {
      const int64_t c = acc[k] >> 32;
      acc[k] -= c * ((int64_t)1 << 32);
      acc[k + 1] += c;
    }
  }
  int h = OR_ACC_DIGITS - 1;
  while (h >= 0 && acc[h] == 0) h--;
  if (h < 0) return 0.0;
  /* 128-bit window of the top four digits, and whether anything lies below */
  unsigned __int128 W = 0;
  for (int k = h; k >= h - 3; k--) W = (W << 32) | (uint64_t)(k >= 0 ? acc[k] : 0);
  int sticky = 0;
  for (int k = h - 4; k >= 0; k--) sticky |= acc[k] != 0;
  int len = 0;
  for (unsigned __int128 t = W; t; t >>= 1) len++;
  const int drop = len - 53;
  uint64_t mant = (uint64_t)(W >> drop);
  const unsigned __int128 rem = W & (((unsigned __int128)1 << drop) - 1);
  const unsigned __int128 half = (unsigned __int128)1 << (drop - 1);
  if (rem > half || (rem == half && (sticky || (mant & 1)))) mant++;
  const double res = ldexp((double)mant, drop + 32 * (h - 3) - 1100);
  return neg ? -res : res;
}

typedef struct {
  int R, C, i0, wrap_x;
} or_lattice;

static or_lattice lattice_of(const or_domain* d) {
  or_lattice L;
  L.i0 = d->poisson_bc == OR_POISSON_PERIODIC ? 0 : 1;
  L.wrap_x = d->poisson_bc == OR_POISSON_PERIODIC;
  L.R = d->nx - 1 - L.i0;
  L.C = d->ny - 1;
  return L;
}

/* The duplicated nodes after a solve: periodic copies (x first, so the corner
 * takes node (0, 0)) and zero x walls. */
static void fill_periodic_nodes(const or_domain* d, double* phi) {
  const int nx = d->nx, ny = d->ny;
  if (d->poisson_bc == OR_POISSON_PERIODIC)
    for (int j = 0; j < ny - 1; j++) phi[IDX(nx - 1, j)] = phi[IDX(0, j)];
  for (int i = 0; i < nx; i++) phi[IDX(i, ny - 1)] = phi[IDX(i, 0)];
  if (d->poisson_bc == OR_POISSON_DIRICHLET_X)
    for (int j = 0; j < ny; j++) phi[IDX(0, j)] = phi[IDX(nx - 1, j)] = 0;
}

/* Subtracts the (correctly rounded) mean of the unknowns' values v[q]. */
static void remove_mean(double* v, long m) {
  const double mean = or_exact_sum(v, m) / (double)m;
  for (long q = 0; q < m; q++) v[q] = v[q] - mean;
}

/* gssolver's sweep on the extension lattices: lexicographic (i outer, j
 * inner) in-place SOR of the same update with wrapped neighbours, the source
 * rho*K (minus its mean when periodic), the L2 residual over the unknowns
 * checked after sweeps 0, 25, 50, ... as sqrt(sum / (nx*ny)). */
static int gs_solve_ext(const or_domain* d, double omega, const double* rho, double* phi, double* err, int* iters) {
  const int nx = d->nx, ny = d->ny;
  const or_lattice L = lattice_of(d);
  const long m = (long)L.R * L.C;
  double dx2 = d->dx * d->dx, dy2 = d->dy * d->dy;
  const double K = (d->L * d->L) / (d->LDe * d->LDe);
  double* src = (double*)malloc(sizeof(double) * m);
  for (int r = 0; r < L.R; r++)
    for (int c = 0; c < L.C; c++) src[(long)r * L.C + c] = rho[IDX(r + L.i0, c)] * K;
  if (L.wrap_x) remove_mean(src, m);
  memset(phi, 0, sizeof(double) * (size_t)nx * ny);
  double L2 = 0;
  int converged = 0;
  double coeff = (2 / dx2) + (2 / dy2);
  int iter;
#define XE(i) ((i) + 1 < nx - 1 || !L.wrap_x ? (i) + 1 : 0)
#define XW(i) ((i) > 0 ? (i) - 1 : nx - 2)
#define YN(j) ((j) + 1 < ny - 1 ? (j) + 1 : 0)
#define YS(j) ((j) > 0 ? (j) - 1 : ny - 2)
  for (iter = 0; iter < d->max_iteration; iter++) {
    for (int r = 0; r < L.R; r++) {
      const int i = r + L.i0;
      for (int j = 0; j < L.C; j++) {
        double phi_new = (1 / coeff) * (src[(long)r * L.C + j] + ((phi[IDX(XE(i), j)] + phi[IDX(XW(i), j)]) / dx2) +
                                        ((phi[IDX(i, YN(j))] + phi[IDX(i, YS(j))]) / dy2));
        phi[IDX(i, j)] = phi[IDX(i, j)] + omega * (phi_new - phi[IDX(i, j)]);
      }
    }
    if (iter % 25 == 0) {
      double sum = 0;
      for (int r = 0; r < L.R; r++) {
        const int i = r + L.i0;
        for (int j = 0; j < L.C; j++) {
          double R = ((phi[IDX(XE(i), j)] - 2 * phi[IDX(i, j)] + phi[IDX(XW(i), j)]) / dx2) +
                     ((phi[IDX(i, YN(j))] - 2 * phi[IDX(i, j)] + phi[IDX(i, YS(j))]) / dy2) + src[(long)r * L.C + j];
          sum += R * R;
        }
      }
      L2 = sqrt(sum / (nx * ny));
      *err = L2;
      if (L2 < d->tolerance) {
        converged = 1;
        break;
      }
    }
  }
#undef XE
#undef XW
#undef YN
#undef YS
  *iters = converged ? iter + 1 : iter;
  if (L.wrap_x) {
    double* u = (double*)malloc(sizeof(double) * m);
    for (int r = 0; r < L.R; r++)
      for (int c = 0; c < L.C; c++) u[(long)r * L.C + c] = phi[IDX(r + L.i0, c)];
    remove_mean(u, m);
    for (int r = 0; r < L.R; r++)
      for (int c = 0; c < L.C; c++) phi[IDX(r + L.i0, c)] = u[(long)r * L.C + c];
    free(u);
  }
  fill_periodic_nodes(d, phi);
  free(src);
  return converged;
}

/* Row q of the extension operator (diagonal -4, wrapped neighbours; beyond
 * the x walls nothing), terms added as the reference's pcg_row adds them:
 * x neighbour below, y neighbour below, the diagonal, y above, x above. */
static double lat_row(const or_lattice* L, const double* v, int r, int c) {
  const int R = L->R, C = L->C;
  double sum = 0;
  if (r > 0) sum += v[(long)(r - 1) * C + c];
  else if (L->wrap_x) sum += v[(long)(R - 1) * C + c];
  sum += v[(long)r * C + (c > 0 ? c - 1 : C - 1)];
  sum += -4 * v[(long)r * C + c];
  sum += v[(long)r * C + (c < C - 1 ? c + 1 : 0)];
  if (r < R - 1) sum += v[(long)(r + 1) * C + c];
  else if (L->wrap_x) sum += v[c];
  return sum;
}

/* pcgsolver's right-hand side -rho*dx^2*K on the extension lattices (minus
 * its mean when periodic), then pcg() of linearalgebra/solvers.h:73-100 as
 * or_pcg_solve runs it; phi with zero mean when periodic; *err =
 * |A x - b| / (nx*ny). */
static int pcg_solve_ext(const or_domain* d, const double* rho, double* phi, double* err, int* iters) {
  const int nx = d->nx, ny = d->ny;
  const or_lattice L = lattice_of(d);
  const long m = (long)L.R * L.C;
  double dx2 = d->dx * d->dx;
  const double K = (d->L * d->L) / (d->LDe * d->LDe);
  double* b = (double*)calloc(m, sizeof(double));
  double* x = (double*)calloc(m, sizeof(double));
  double* r = (double*)calloc(m, sizeof(double));
  double* w = (double*)calloc(m, sizeof(double));
  double* v = (double*)calloc(m, sizeof(double));
  double* u = (double*)calloc(m, sizeof(double));
  for (int rr = 0; rr < L.R; rr++)
    for (int c = 0; c < L.C; c++) b[(long)rr * L.C + c] = -rho[IDX(rr + L.i0, c)] * dx2 * K;
  if (L.wrap_x) remove_mean(b, m);
  for (long k = 0; k < m; k++) r[k] = b[k] - 0.0;
  double minv = 1.0 / -4.0;
  for (long k = 0; k < m; k++) { w[k] = minv * r[k]; v[k] = w[k]; }
  double alpha = dot(w, r, m);
  /* min(m*m, max_iteration) as pcg() caps it, with m*m in 64 bits (the
   * reference's 32-bit product wraps negative for lattices this size). */
  const long long cap = (long long)m * m;
  int maxit = cap < d->max_iteration ? (int)cap : d->max_iteration;
  int it = 0;
  for (it = 0; it < maxit; it++) {
    if (sqrt(dot(r, r, m)) < d->tolerance) break;
    for (int rr = 0; rr < L.R; rr++)
      for (int c = 0; c < L.C; c++) u[(long)rr * L.C + c] = lat_row(&L, v, rr, c);
    double t = alpha / dot(v, u, m);
    for (long k = 0; k < m; k++) x[k] = x[k] + v[k] * t;
    for (long k = 0; k < m; k++) r[k] = r[k] - u[k] * t;
    for (long k = 0; k < m; k++) w[k] = minv * r[k];
    double beta = dot(w, r, m);
    double s = beta / alpha;
    for (long k = 0; k < m; k++) v[k] = w[k] + v[k] * s;
    alpha = beta;
  }
  double e2 = 0;
  for (int rr = 0; rr < L.R; rr++)
    for (int c = 0; c < L.C; c++) {
      double e = lat_row(&L, x, rr, c) - b[(long)rr * L.C + c];
      e2 += e * e;
    }
  *err = sqrt(e2) / ((long)nx * ny);
  *iters = it;
  if (L.wrap_x) remove_mean(x, m);
  memset(phi, 0, sizeof(double) * (size_t)nx * ny);
  for (int rr = 0; rr < L.R; rr++)
    for (int c = 0; c < L.C; c++) phi[IDX(rr + L.i0, c)] = x[(long)rr * L.C + c];
  fill_periodic_nodes(d, phi);
  free(b); free(x); free(r); free(w); free(v); free(u);
  return it < maxit;
}

/* ------------------------------------------------------------ solvers --- */
/* FieldSolve::gssolver (src/field.cpp:70-139): cold start, phi = 0 on every
 * edge, lexicographic (i outer, j inner) in-place SOR, L2 residual check
 * after sweeps 0, 25, 50, ... */
int or_gs_solve(const or_domain* d, double omega, const double* rho, double* phi, double* err, int* iters) {
  if (d->poisson_bc != OR_POISSON_REFERENCE) return gs_solve_ext(d, omega, rho, phi, err, iters);
  const int nx = d->nx, ny = d->ny;
  double dx2 = d->dx * d->dx, dy2 = d->dy * d->dy;
  memset(phi, 0, sizeof(double) * (size_t)nx * ny);
  double L2 = 0;
  int converged = 0;
  double coeff = (2 / dx2) + (2 / dy2);
  int iter;
  for (iter = 0; iter < d->max_iteration; iter++) {
    for (int i = 1; i < nx - 1; i++) {
      for (int j = 1; j < ny - 1; j++) {
        double phi_new = (1 / coeff) * (rho[IDX(i, j)] * ((d->L * d->L) / (d->LDe * d->LDe)) +
                                        ((phi[IDX(i + 1, j)] + phi[IDX(i - 1, j)]) / dx2) +
                                        ((phi[IDX(i, j + 1)] + phi[IDX(i, j - 1)]) / dy2));
        phi[IDX(i, j)] = phi[IDX(i, j)] + omega * (phi_new - phi[IDX(i, j)]);
      }
    }
    if (iter % 25 == 0) {
      double sum = 0;
      for (int i = 1; i < nx - 1; i++) {
        for (int j = 1; j < ny - 1; j++) {
          double R = ((phi[IDX(i + 1, j)] - 2 * phi[IDX(i, j)] + phi[IDX(i - 1, j)]) / dx2) +
                     ((phi[IDX(i, j + 1)] - 2 * phi[IDX(i, j)] + phi[IDX(i, j - 1)]) / dy2) +
                     (rho[IDX(i, j)]) * ((d->L * d->L) / (d->LDe * d->LDe));
          sum += R * R;
        }
      }
      L2 = sqrt(sum / (nx * ny));
      *err = L2;
      if (L2 < d->tolerance) {
        converged = 1;
        break;
      }
    }
  }
  *iters = converged ? iter + 1 : iter;
  return converged;
}

/* Row k of the reference's dense operator (src/field.cpp:221-232: row = k/nx,
 * col = k%nx, diagonal -4, off-diagonals 1) times v.  The dense product of
 * linearalgebra/linalg.h:387-432 adds A(k,j)*v(j) for j = 0..n-1 starting from
 * 0; the zero entries leave the sum unchanged, so the result is the stencil
 * terms added in increasing column order. */
/* FieldSolve::gsfluidsolver (src/field.cpp:7-68), "gshybrid": the SOR sweep
 * of gssolver with Boltzmann electrons, source (rho - exp(phi)) * K, after
 * setting rho on the edges (bottom 0, top 10000 * eV/(k_B EV_to_K), then left
 * and right 0, in that order); the residual is checked every 50 sweeps.  rho
 * is modified in place, as domain.rho is. */
int or_gsfluid_solve(const or_domain* d, double* rho, double* phi, double* err, int* iters) {
  const int nx = d->nx, ny = d->ny;
  double dx2 = d->dx * d->dx, dy2 = d->dy * d->dy;
  memset(phi, 0, sizeof(double) * (size_t)nx * ny);
  double L2 = 0;
  int converged = 0;
  double coeff = (2 / dx2) + (2 / dy2);
  for (int i = 0; i < nx; i++) {
    rho[IDX(i, 0)] = 0;
    rho[IDX(i, ny - 1)] = 10000 * (OR_QE / (OR_K_B * (OR_QE / OR_K_B)));
  }
  for (int i = 0; i < ny; i++) {
    rho[IDX(0, i)] = 0;
    rho[IDX(nx - 1, i)] = 0;
  }
  const double K = (d->L * d->L) / (d->LDe * d->LDe);
  int iter;
  for (iter = 0; iter < d->max_iteration; iter++) {
    for (int i = 1; i < nx - 1; i++) {
      for (int j = 1; j < ny - 1; j++) {
        double phi_new = (1 / coeff) * ((rho[IDX(i, j)] - exp(phi[IDX(i, j)])) * K +
                                        ((phi[IDX(i + 1, j)] + phi[IDX(i - 1, j)]) / dx2) +
                                        ((phi[IDX(i, j + 1)] + phi[IDX(i, j - 1)]) / dy2));
        phi[IDX(i, j)] = phi[IDX(i, j)] + 1.4 * (phi_new - phi[IDX(i, j)]);
      }
    }
    if (iter % 50 == 0) {
      double sum = 0;
      for (int i = 1; i < nx - 1; i++) {
        for (int j = 1; j < ny - 1; j++) {
          double R = ((phi[IDX(i + 1, j)] - 2 * phi[IDX(i, j)] + phi[IDX(i - 1, j)]) / dx2) +
                     ((phi[IDX(i, j + 1)] - 2 * phi[IDX(i, j)] + phi[IDX(i, j - 1)]) / dy2) +
                     (rho[IDX(i, j)] - exp(phi[IDX(i, j)])) * K;
          sum += R * R;
        }
      }
      L2 = sqrt(sum / (nx * ny));
      *err = L2;
      if (L2 < d->tolerance) {
        converged = 1;
        break;
      }
    }
  }
  *iters = converged ? iter + 1 : iter;
  return converged;
}

/* The dense 5-point matrix of nrpcgsolver (src/field.cpp:150-161: row k / nx,
 * column k % nx of the flattened vector, diagonal diag[k]) times v, summed in
 * ascending column order like Matrix::operator*(vec) (linearalgebra/linalg.h:
 * 388-430, whose zero entries leave the sum unchanged). */
static void nr_matvec(int nx, int ny, const double* diag, double cdiag, const double* v, double* out) {
  const long n = (long)nx * ny;
  for (long k = 0; k < n; k++) {
    const long row = k / nx, col = k % nx;
    double sum = 0;
    if (row > 0) sum += 1.0 * v[k - nx];
    if (col > 0) sum += 1.0 * v[k - 1];
    sum += (diag ? diag[k] : cdiag) * v[k];
    if (col < nx - 1) sum += 1.0 * v[k + 1];
    if (row < ny - 1) sum += 1.0 * v[k + nx];
    out[k] = sum;
  }
}

static double nr_dot(const double* a, const double* b, long n) {  /* vec::operator*, serial */
  double r = 0;
  for (long i = 0; i < n; i++) r += a[i] * b[i];
  return r;
}

/* FieldSolve::nrpcgsolver (src/field.cpp:141-210), "hybrid": ten Newton steps
 * on A x - rhovec with rhovec += exp(x) K every step (the reference accumulates
 * it) and J = A - diag(exp(x)), each solved by cg (linearalgebra/solvers.h:
 * 33-69, tolerance 1e-4, at most min(n, 10000) iterations, from x = 0).
 * Returns the CG iterations in total; domain.error is set to 0. */
long or_nrpcg_solve(const or_domain* d, const double* rho, double* phi, double* err) {
  const int nx = d->nx, ny = d->ny;
  const long n = (long)nx * ny;
  const double dx2 = d->dx * d->dx;
  const double K = (d->L * d->L) / (d->LDe * d->LDe);
  double* rhovec = calloc((size_t)n, sizeof(double));
  double* x = calloc((size_t)n, sizeof(double));
  double* F = calloc((size_t)n, sizeof(double));
  double* J = calloc((size_t)n, sizeof(double));
  double* y = calloc((size_t)n, sizeof(double));
  double* r = calloc((size_t)n, sizeof(double));
  double* p = calloc((size_t)n, sizeof(double));
  double* Ap = calloc((size_t)n, sizeof(double));
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      double v = -rho[IDX(i, j)] * dx2 * K;
      if (j == 0 || j == ny - 1 || i == 0 || i == nx - 1) v = 0;
      rhovec[IDX(i, j)] = v;
    }
  long total = 0;
  const long maxit = n < 10000 ? n : 10000;
  for (int it = 0; it < 10; it++) {
    for (long k = 0; k < n; k++) rhovec[k] = rhovec[k] + exp(x[k]) * K;
    nr_matvec(nx, ny, 0, -4, x, F);
    for (long k = 0; k < n; k++) {
      F[k] = F[k] - rhovec[k];
      J[k] = -4 - exp(x[k]);
    }
    /* cg(J, 0, F): r0 = F - J*0 = F */
    for (long k = 0; k < n; k++) {
      y[k] = 0;
      r[k] = F[k] - 0.0;
      p[k] = r[k];
    }
    double r02 = nr_dot(r, r, n);
    for (long i = 0; i < maxit; i++) {
      if (sqrt(r02) < 1e-4) break;
      nr_matvec(nx, ny, J, 0, p, Ap);
      double pAp = nr_dot(p, Ap, n);
      double alpha = r02 / pAp;
      for (long k = 0; k < n; k++) {
        y[k] = y[k] + p[k] * alpha;
        r[k] = r[k] - Ap[k] * alpha;
      }
      double r12 = nr_dot(r, r, n);
      double beta = r12 / r02;
      for (long k = 0; k < n; k++) p[k] = r[k] + p[k] * beta;
      r02 = r12;
      total++;
    }
    for (long k = 0; k < n; k++) x[k] = x[k] - y[k];
  }
  memcpy(phi, x, sizeof(double) * (size_t)n);
  *err = 0;
  free(rhovec); free(x); free(F); free(J); free(y); free(r); free(p); free(Ap);
  return total;
}

static double pcg_row(long k, int nx, int ny, const double* v) {
  long row = k / nx, col = k % nx;
  double sum = 0;
  if (row > 0) sum += v[k - nx];
  if (col > 0) sum += v[k - 1];
  sum += -4 * v[k];
  if (col < nx - 1) sum += v[k + 1];
  if (row < ny - 1) sum += v[k + nx];
  return sum;
}

static double dot(const double* a, const double* b, long n) {
  double r = 0;
  for (long i = 0; i < n; i++) r += a[i] * b[i];
  return r;
}

/* FieldSolve::pcgsolver (src/field.cpp:212-264) + pcg (linearalgebra/
 * solvers.h:73-100) with the Jacobi preconditioner of linearalgebra/
 * function.h:97-105 (1/(-4) on the diagonal).  The iteration cap is
 * min(n*n, max_iteration) with n*n in 32-bit int arithmetic, as the reference. */
int or_pcg_solve(const or_domain* d, const double* rho, double* phi, double* err, int* iters) {
  if (d->poisson_bc != OR_POISSON_REFERENCE) return pcg_solve_ext(d, rho, phi, err, iters);
  const int nx = d->nx, ny = d->ny;
  const long n = (long)nx * ny;
  double dx2 = d->dx * d->dx;
  double* b = (double*)calloc(n, sizeof(double));
  double* x = (double*)calloc(n, sizeof(double));
  double* r = (double*)calloc(n, sizeof(double));
  double* w = (double*)calloc(n, sizeof(double));
  double* v = (double*)calloc(n, sizeof(double));
  double* u = (double*)calloc(n, sizeof(double));
  double K = (d->L * d->L) / (d->LDe * d->LDe);
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) b[IDX(i, j)] = -rho[IDX(i, j)] * dx2 * K;
  for (int i = 0; i < nx; i++) { b[IDX(i, 0)] = 0; b[IDX(i, ny - 1)] = 0; }
  for (int j = 0; j < ny; j++) { b[IDX(0, j)] = 0; b[IDX(nx - 1, j)] = 0; }
  /* flatten (linearalgebra/function.h:155-168) keeps index i*ny + j. */
  for (long k = 0; k < n; k++) r[k] = b[k] - 0.0;
  double minv = 1.0 / -4.0;
  for (long k = 0; k < n; k++) { w[k] = minv * r[k]; v[k] = w[k]; }
  double alpha = dot(w, r, n);
  int cap = (int)((uint32_t)n * (uint32_t)n);
  int maxit = cap < d->max_iteration ? cap : d->max_iteration;
  int it = 0;
  for (it = 0; it < maxit; it++) {
    if (sqrt(dot(r, r, n)) < d->tolerance) break;
    for (long k = 0; k < n; k++) u[k] = pcg_row(k, nx, ny, v);
    double t = alpha / dot(v, u, n);
    for (long k = 0; k < n; k++) x[k] = x[k] + v[k] * t;
    for (long k = 0; k < n; k++) r[k] = r[k] - u[k] * t;
    for (long k = 0; k < n; k++) w[k] = minv * r[k];
    double beta = dot(w, r, n);
    double s = beta / alpha;
    for (long k = 0; k < n; k++) v[k] = w[k] + v[k] * s;
    alpha = beta;
  }
  double e2 = 0;
  for (long k = 0; k < n; k++) {
    double e = pcg_row(k, nx, ny, x) - b[k];
    e2 += e * e;
  }
  *err = sqrt(e2) / n;
  *iters = it;
  memcpy(phi, x, sizeof(double) * n);
  free(b); free(x); free(r); free(w); free(v); free(u);
  return it < maxit;
}

/* FieldSolve::CalculateEfield (src/field.cpp:276-330).  The edge formulas
 * follow bc as there (periodic central for pbc, one-sided otherwise); with a
 * Poisson extension they follow the field's boundary instead: periodic
 * directions take the periodic central formula, the x walls of dirichlet_x
 * the one-sided one. */
void or_efield(const or_domain* d, const double* phi, double* efx, double* efy) {
  const int nx = d->nx, ny = d->ny;
  const double dx = d->dx, dy = d->dy;
  int x_periodic = d->bc == OR_PBC, x_onesided = d->bc == OR_OPEN || d->bc == OR_REFLECTIVE;
  int y_periodic = x_periodic, y_onesided = x_onesided;
  if (d->poisson_bc == OR_POISSON_PERIODIC) {
    x_periodic = y_periodic = 1;
    x_onesided = y_onesided = 0;
  } else if (d->poisson_bc == OR_POISSON_DIRICHLET_X) {
    x_periodic = 0; x_onesided = 1;
    y_periodic = 1; y_onesided = 0;
  }
  for (int i = 1; i < nx - 1; i++)
    for (int j = 0; j < ny; j++) efx[IDX(i, j)] = -(phi[IDX(i + 1, j)] - phi[IDX(i - 1, j)]) / (2 * dx);
  if (x_onesided) {
    for (int j = 0; j < ny; j++) {
      efx[IDX(0, j)] = -(phi[IDX(1, j)] - phi[IDX(0, j)]) / dx;
      efx[IDX(nx - 1, j)] = -(phi[IDX(nx - 1, j)] - phi[IDX(nx - 2, j)]) / dx;
    }
  }
  if (x_periodic) {
    for (int j = 0; j < ny; j++) {
      efx[IDX(0, j)] = -(phi[IDX(1, j)] - phi[IDX(nx - 2, j)]) / (2 * dx);
      efx[IDX(nx - 1, j)] = efx[IDX(0, j)];
    }
  }
  for (int i = 0; i < nx; i++)
    for (int j = 1; j < ny - 1; j++) efy[IDX(i, j)] = -(phi[IDX(i, j + 1)] - phi[IDX(i, j - 1)]) / (2 * dy);
  if (y_onesided) {
    for (int i = 0; i < nx; i++) {
      efy[IDX(i, 0)] = -(phi[IDX(i, 1)] - phi[IDX(i, 0)]) / dy;
      efy[IDX(i, ny - 1)] = -(phi[IDX(i, ny - 1)] - phi[IDX(i, ny - 2)]) / dy;
    }
  }
  if (y_periodic) {
    for (int i = 0; i < nx; i++) {
      efy[IDX(i, 0)] = -(phi[IDX(i, 1)] - phi[IDX(i, ny - 2)]) / (2 * dy);
      efy[IDX(i, ny - 1)] = efy[IDX(i, 0)];
    }
  }
}

/* ------------------------------------------------------------- push --- */
/* Domain::Interpolate (src/domain.cpp:231-255). */
static double interp(const or_domain* d, double lx, double ly, const double* f) {
  const int ny = d->ny;
  int i = (int)lx, j = (int)ly;
  double di = lx - i, dj = ly - j;
  if (d->shape == OR_NGP) return f[IDX((int)round(lx), (int)round(ly))];
  return f[IDX(i, j)] * (1 - di) * (1 - dj) + f[IDX(i + 1, j)] * (di) * (1 - dj) + f[IDX(i, j + 1)] * (1 - di) * (dj) +
         f[IDX(i + 1, j + 1)] * (di) * (dj);
}

/* Species::Push_species_serial (src/species.cpp:29-170), erasing particles
 * that end inside a conductor (:80-97, :108-121, :150-165). */
long or_push_c(const or_domain* d, double mass, double charge, int sub_cycle, double* part, long n,
               const double* efx, const double* efy, const double* grids, int ng, int circles_live);
long or_push(const or_domain* d, double mass, double charge, int sub_cycle, double* part, long n,
             const double* efx, const double* efy) {
  return or_push_c(d, mass, charge, sub_cycle, part, n, efx, efy, 0, 0, 0);
}

long or_push_c(const or_domain* d, double mass, double charge, int sub_cycle, double* part, long n,
               const double* efx, const double* efy, const double* grids, int ng, int circles_live) {
  long out = 0;
  for (long p = 0; p < n; p++) {
    double* q = part + 5 * p;
    double qm = charge / mass;
    double lx = (q[0] - d->x0) / d->dx;
    double ly = (q[1] - d->y0) / d->dy;
    double ex = interp(d, lx, ly, efx);
    double ey = interp(d, lx, ly, efy);
    double K = (d->density * OR_QE * d->L) / (OR_EPS_0 * d->W * d->vel_norm);
    q[2] += qm * K * ex * (d->DT * sub_cycle);
    q[3] += qm * K * ey * (d->DT * sub_cycle);
    double c = (d->vel_norm) / (d->L * d->W);
    q[0] += c * q[2] * (d->DT * sub_cycle);
    q[1] += c * q[3] * (d->DT * sub_cycle);
    if (d->bc == OR_PBC) {
      if (q[0] < d->x0) q[0] = q[0] + d->Lx;
      else if (q[0] >= d->x0 + d->Lx) q[0] = q[0] - d->Lx;
      if (q[1] < d->x0) q[1] = q[1] + d->Ly;
      else if (q[1] >= d->x0 + d->Ly) q[1] = q[1] - d->Ly;
    } else if (d->bc == OR_OPEN) {
      if (q[0] < d->x0 || q[0] >= d->x0 + d->Lx || q[1] < d->x0 || q[1] >= d->x0 + d->Ly) continue;
    } else if (d->bc == OR_REFLECTIVE) {
      if (q[0] < d->x0) { q[0] = d->x0 + (d->x0 - q[0]); q[2] = -q[2]; }
      else if (q[0] >= d->x0 + d->Lx) { q[0] = d->x0 + d->Lx - (q[0] - (d->x0 + d->Lx)); q[2] = -q[2]; }
      if (q[1] < d->x0) { q[1] = d->x0 + (d->x0 - q[1]); q[3] = -q[3]; }
      else if (q[1] >= d->x0 + d->Ly) { q[1] = d->x0 + d->Ly - (q[1] - (d->x0 + d->Ly)); q[3] = -q[3]; }
    }
    if (ng && or_in_conductors(grids, ng, circles_live, q[0], q[1])) continue;
    if (out != p) memmove(part + 5 * out, q, 5 * sizeof(double));
    out++;
  }
  return out;
}

/* Species::Rewind_species (src/species.cpp:229-246). */
void or_rewind(const or_domain* d, double mass, double charge, double* part, long n, const double* efx,
               const double* efy) {
  for (long p = 0; p < n; p++) {
    double* q = part + 5 * p;
    double qm = charge / mass;
    double lx = (q[0] - d->x0) / d->dx;
    double ly = (q[1] - d->y0) / d->dy;
    double ex = interp(d, lx, ly, efx);
    double ey = interp(d, lx, ly, efy);
    double K = (d->density * OR_QE * d->L) / (OR_EPS_0 * d->W * d->vel_norm);
    q[2] -= 0.5 * qm * K * ex * d->DT;
    q[3] -= 0.5 * qm * K * ey * d->DT;
  }
}

/* ------------------------------------------------------------- MCC --- */
/* e-/Ar fits of src/cross_section.cpp:4-39 (energy in eV, result in m^2). */
double or_cs_elastic(double energy, int enabled) {
  if (!enabled) return 0.0;
  return (1e-20 * fabs(6.0 / pow(1.0 + (energy / 0.1) + pow(energy / 0.6, 2.0), 3.3) -
                       1.1 * pow(energy, 1.4) / (1.0 + pow(energy / 15.0, 1.2)) /
                           sqrt(1.0 + pow(energy / 5.5, 2.5) + pow(energy / 60.0, 4.1)) +
                       0.05 / pow(1.0 + energy / 10.0, 2.0) + 0.01 * pow(energy, 3.0) / (1.0 + pow(energy / 12.0, 6.0))));
}

double or_cs_excitation(double energy, int enabled) {
  if (!enabled) return 0.0;
  if (energy > OR_E_EXC_TH) {
    return (1e-20 * (0.034 * pow(energy - OR_E_EXC_TH, 1.1) * (1.0 + pow(energy / 15.0, 2.8)) /
                         (1.0 + pow(energy / 23.0, 5.5)) +
                     0.023 * (energy - OR_E_EXC_TH) / pow(1.0 + energy / 80.0, 1.9)));
  }
  return 0.0;
}

double or_cs_ionization(double energy, int enabled) {
  if (!enabled) return 0.0;
  if (energy > OR_E_ION_TH) {
    return (1e-20 * (970.0 * (energy - OR_E_ION_TH) / pow(70.0 + energy, 2.0) +
                     0.06 * pow(energy - OR_E_ION_TH, 2.0) * exp(-energy / 9)));
  }
  return 0.0;
}

/* CollisionHandler::set_electron_cross_sections / calc_total_cross_sections
 * (src/collision.cpp:21-42): energy[0] = DE_CS, energy[i] = DE_CS * i. */
void or_cs_tables(const or_domain* d, double* tot, double* ela, double* exc, double* ion) {
  for (long i = 0; i < OR_CS_RANGES; i++) {
    double e = i == 0 ? OR_DE_CS : OR_DE_CS * (int)i;
    ela[i] = or_cs_elastic(e, d->elastic);
    exc[i] = or_cs_excitation(e, d->excitation);
    ion[i] = or_cs_ionization(e, d->ionization);
    tot[i] = (ela[i] + exc[i] + ion[i]) * d->gas_density;
  }
}

typedef struct {
  or_rng* rng;
  const double* u;
  int k, stride;
} draw_src;

static double draw(draw_src* s) {
  if (s->rng) return or_rng_uniform(s->rng);
  return s->u[s->k++];
}

static double draw_sample_vel(draw_src* s, double mass, double temp) {
  double v_th = sqrt(2 * OR_K_B * temp * (OR_QE / OR_K_B) / mass);
  double u1 = draw(s);
  double u2 = draw(s);
  double u3 = draw(s);
  return v_th * sqrt(2) * (u1 + u2 + u3 - 1.5);
}

void or_table_log(or_table* t, long n, double e_min, double e_max) {
  t->kind = 1;
  t->n = n;
  t->e_min = e_min;
  t->e_max = e_max;
  t->log_emin = log(e_min);
  t->inv_dlog = (n - 1) / (log(e_max) - log(e_min));
}

typedef struct {
  double tot, ela, exc, ion;
} sigma4;

static sigma4 table_at(const or_table* t, double energy) {
  sigma4 s;
  if (t->kind == 0) {
    int idx = (int)(energy / t->de + 0.5);
    if (idx > (int)t->n - 1) idx = (int)t->n - 1;
    s.tot = t->tot[idx];
    s.ela = t->ela[idx];
    s.exc = t->exc[idx];
    s.ion = t->ion[idx];
  } else {
    double e = fmin(fmax(energy, t->e_min), t->e_max);
    double uu = (log(e) - t->log_emin) * t->inv_dlog;
    int i = (int)uu;
    if (i > (int)t->n - 2) i = (int)t->n - 2;
    if (i < 0) i = 0;
    double f = uu - i;
    s.ela = t->ela[i] * (1 - f) + t->ela[i + 1] * f;
    s.exc = t->exc[i] * (1 - f) + t->exc[i + 1] * f;
    s.ion = t->ion[i] * (1 - f) + t->ion[i + 1] * f;
    s.tot = t->tot[i] * (1 - f) + t->tot[i + 1] * f;
  }
  return s;
}

long or_mcc(const or_domain* d, const double* tot, const double* ela, const double* exc, const double* ion,
            double* e_part, long* n_e, long e_cap, double ion_mass, double ion_temp, double* i_part, long* n_i,
            long i_cap, int mode, or_rng* rng, const double* u, int ustride, int* kinds) {
  or_table t;
  memset(&t, 0, sizeof(t));
  t.kind = 0;
  t.n = OR_CS_RANGES;
  t.de = OR_DE_CS;
  t.tot = tot;
  t.ela = ela;
  t.exc = exc;
  t.ion = ion;
  return or_mcc_table(d, &t, e_part, n_e, e_cap, ion_mass, ion_temp, i_part, n_i, i_cap, mode, rng, u, ustride,
                      kinds);
}

long or_mcc_table(const or_domain* d, const or_table* tab, double* e_part, long* n_e, long e_cap, double ion_mass,
                  double ion_temp, double* i_part, long* n_i, long i_cap, int mode, or_rng* rng, const double* u,
                  int ustride, int* kinds) {
  long ne0 = *n_e;
  long ncoll = 0;
  const double F1 = OR_ME / (OR_ME + ion_mass);
  const double F2 = ion_mass / (OR_ME + ion_mass);
  const double vn = d->vel_norm;
  for (long p = 0; p < ne0; p++) {
    draw_src src = {mode == 0 ? rng : NULL, mode == 0 ? NULL : u + (long)p * ustride, 0, ustride};
    double* q = e_part + 5 * p;
    if (kinds) kinds[p] = 0;
    double v_sqr = (q[2] * q[2] + q[3] * q[3] + q[4] * q[4]) * vn * vn;
    double velocity = sqrt(v_sqr);
    double energy = (0.5 * OR_ME * v_sqr) / OR_EV;
    sigma4 sg = table_at(tab, energy);
    double nu = sg.tot * velocity;
    double p_coll = 1 - exp(-nu * (d->DT / d->W));
    if (!(p_coll > draw(&src))) continue;
    ncoll++;
    /* collision_electron, src/collision.cpp:60-188 */
    double gx = q[2], gy = q[3], gz = q[4];
    double g = sqrt(gx * gx + gy * gy + gz * gz);
    double wx = F1 * q[2], wy = F1 * q[3], wz = F1 * q[4];
    double theta, phi, chi, eta;
    if (gx == 0) theta = 0.5 * OR_PI;
    else theta = atan2(sqrt(gy * gy + gz * gz), gx);
    if (gy == 0) phi = gz > 0 ? 0.5 * OR_PI : -0.5 * OR_PI;
    else phi = atan2(gz, gy);
    double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
    double t0 = sg.ela;
    double t1 = t0 + sg.exc;
    double t2 = t1 + sg.ion;
    if (draw(&src) < (t0 / t2)) {
      if (kinds) kinds[p] = 1;
      chi = acos(1.0 - 2.0 * draw(&src));
      eta = 2 * OR_PI * draw(&src);
    } else if (draw(&src) < (t1 / t2)) {
      if (kinds) kinds[p] = 2;
      double en = 0.5 * OR_ME * g * g * vn * vn;
      en = fabs(en - OR_E_EXC_TH * OR_EV);
      g = sqrt(2.0 * en / OR_ME);
      g = g / vn;
      chi = acos(1.0 - 2.0 * draw(&src));
      eta = 2 * OR_PI * draw(&src);
    } else {
      if (kinds) kinds[p] = 3;
      double en = 0.5 * OR_ME * g * g * vn * vn;
      en = fabs(en - OR_E_ION_TH * OR_EV);
      double e_ej = 10.0 * tan(draw(&src) * atan(en / OR_EV / 20.0)) * OR_EV;
      double e_sc = fabs(en - e_ej);
      g = sqrt(2.0 * e_sc / OR_ME);
      double g2 = sqrt(2.0 * e_ej / OR_ME);
      g = g / vn;
      g2 = g2 / vn;
      chi = acos(sqrt(e_sc / en));
      double chi2 = acos(sqrt(e_ej / en));
      eta = 2 * OR_PI * draw(&src);
      double eta2 = eta + OR_PI;
      double sc = sin(chi2), cc = cos(chi2), se = sin(eta2), ce = cos(eta2);
      double hx = g2 * (ct * cc - st * sc * ce);
      double hy = g2 * (st * cp * cc + ct * cp * sc * ce - sp * sc * se);
      double hz = g2 * (st * sp * cc + ct * sp * sc * ce + cp * sc * se);
      if (*n_e >= e_cap || *n_i >= i_cap) return -1;
      double* ne = e_part + 5 * (*n_e);
      ne[0] = q[0]; ne[1] = q[1];
      ne[2] = (wx + F2 * hx); ne[3] = (wy + F2 * hy); ne[4] = (wz + F2 * hz);
      (*n_e)++;
      /* Particle(xe, ye, SampleVel, SampleVel, SampleVel): GCC evaluates the
       * three constructor arguments right to left (pinned against
       * oracle/_ref), so vz takes the first three draws.  The ion velocity is
       * left in m/s, unnormalised, as in the reference. */
      double ivz = draw_sample_vel(&src, ion_mass, ion_temp);
      double ivy = draw_sample_vel(&src, ion_mass, ion_temp);
      double ivx = draw_sample_vel(&src, ion_mass, ion_temp);
      double* ni = i_part + 5 * (*n_i);
      ni[0] = q[0]; ni[1] = q[1]; ni[2] = ivx; ni[3] = ivy; ni[4] = ivz;
      (*n_i)++;
    }
    double sc = sin(chi), cc = cos(chi), se = sin(eta), ce = cos(eta);
    gx = g * (ct * cc - st * sc * ce);
    gy = g * (st * cp * cc + ct * cp * sc * ce - sp * sc * se);
    gz = g * (st * sp * cc + ct * sp * sc * ce + cp * sc * se);
    q[2] = wx + F2 * gx;
    q[3] = wy + F2 * gy;
    q[4] = wz + F2 * gz;
  }
  return ncoll;
}

/* ------------------------------------------------------- diagnostics --- */
/* Species::Compute_KE (src/species.cpp:248-271). */
void or_ke(const or_domain* d, const double* part, long n, double mass, double spwt, double norm_temp,
           double norm_spwt, int norm_num, double* out3) {
  double k0 = 0, k1 = 0, k2 = 0;
  const double vn = d->vel_norm;
  for (long p = 0; p < n; p++) {
    const double* q = part + 5 * p;
    k0 += (q[2] * q[2]) * (vn) * (vn);
    k1 += (q[3] * q[3]) * (vn) * (vn);
    k2 += (q[4] * q[4]) * (vn) * (vn);
  }
  k0 *= 0.5 * (spwt * mass);
  k1 *= 0.5 * (spwt * mass);
  k2 *= 0.5 * (spwt * mass);
  double Th = (norm_temp * OR_EV) * (norm_spwt) * norm_num;
  out3[0] = k0 / Th;
  out3[1] = k1 / Th;
  out3[2] = k2 / Th;
}

/* Species::Compute_Momentum (src/species.cpp:273-297). */
void or_momentum(const or_domain* d, const double* part, long n, double mass, double spwt, double norm_temp,
                 double norm_spwt, int norm_num, double* out3) {
  double p0 = 0, p1 = 0, p2 = 0;
  const double vn = d->vel_norm;
  for (long p = 0; p < n; p++) {
    const double* q = part + 5 * p;
    p0 += (q[2]) * vn;
    p1 += (q[3]) * vn;
    p2 += (q[4]) * vn;
  }
  p0 *= (spwt * mass);
  p1 *= (spwt * mass);
  p2 *= (spwt * mass);
  double Thp = sqrt(norm_temp * OR_EV / OR_ME) * norm_spwt * norm_num * OR_ME;
  out3[0] = p0 / Thp;
  out3[1] = p1 / Thp;
  out3[2] = p2 / Thp;
}

/* Domain::Compute_PE (src/domain.cpp:266-286). */
double or_pe(const or_domain* d, const double* efx, const double* efy, double norm_temp, double norm_spwt,
             int norm_num) {
  const int nx = d->nx, ny = d->ny;
  double pe = 0;
  double unnorm = (d->density * OR_QE * d->L) / OR_EPS_0;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      double ef2 = efx[IDX(i, j)] * efx[IDX(i, j)] + efy[IDX(i, j)] * efy[IDX(i, j)];
      pe += ef2 * (d->L * d->L);
    }
  double pe_norm = 0.5 * OR_EPS_0 * pe * unnorm * unnorm;
  double Th = (norm_temp * OR_EV) * norm_spwt * norm_num;
  pe_norm /= Th;
  return pe_norm;
}
