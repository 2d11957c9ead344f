/* FP64 CPU restatement of the reference's Monte Carlo energy path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle). Loaded by tests/, the smoke check
 * and bench.py's CPU-baseline leg; never by the product.
 *
 * Each function names the reference lines it restates. Arithmetic is kept in
 * the reference's evaluation order wherever the result feeds a comparison
 * (rejection loops, cut-offs, the Metropolis test), so the draw sequence and
 * accept/reject decisions match the reference for the same mt19937 stream.
 * The reciprocal Ewald term is the one deliberate rewrite: the reference sums
 * (4 pi lB q_i q_j / V) sum_k e^{-k^2/4a}/k^2 cos(k.r_ij) over pairs
 * (potential_ewald_coul.cc:198-225); here it is (4 pi lB / V) sum over the
 * half k-space of e^{-k^2/4a}/k^2 |S(k)|^2 on the identical k-set, which is
 * the same quantity.
 */
#include "plum_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* utilities/constants.h:5-62 */
#define K_EWALD_CUTOFF 1e-7
#define K_VERY_LARGE 1e8
#define K_PI 3.14159265359
#define K213 1.25992104989
#define K216 1.12246204831
#define K_DI_CORRECTION 3
#define K_NO_MOVE_TYPE 5
#define K_MED_SMALL 1e-4
#define MAXT 64
/* M_PI as <cmath> defines it; the crankshaft angle uses it (molecule.cc:247). */
#define M_PI_LIBM 3.14159265358979323846

/* ------------------------------------------------------------------ mt19937 */
/* Matsumoto & Nishimura (1998) MT19937 with the standard initialisation and
 * tempering; std::mt19937 (used by the reference, simulation.h:148) is this
 * generator. */
typedef struct {
  uint32_t mt[624];
  int idx;
} mt_t;

static void mt_seed(mt_t* g, uint32_t s) {
  g->mt[0] = s;
  for (int i = 1; i < 624; i++)
    g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
  g->idx = 624;
}

static uint32_t mt_next(mt_t* g) {
  if (g->idx >= 624) {
    for (int i = 0; i < 624; i++) {
      uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
      uint32_t v = g->mt[(i + 397) % 624] ^ (y >> 1);
      if (y & 1u) v ^= 0x9908b0dfu;
      g->mt[i] = v;
    }
    g->idx = 0;
  }
  uint32_t y = g->mt[g->idx++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

void po_mt19937(uint32_t seed, long n, uint32_t* out) {
  mt_t g;
  mt_seed(&g, seed);
  for (long i = 0; i < n; i++) out[i] = mt_next(&g);
}

/* Draw source: the internal generator or a recorded stream. */
typedef struct {
  mt_t* g;
  const uint32_t* s;
  long n, pos;
  int overrun;
} rng_t;

static uint32_t rng_u32(rng_t* r) {
  if (r->s) {
    if (r->pos >= r->n) {
      r->overrun = 1;
      return 0;
    }
    return r->s[r->pos++];
  }
  r->pos++;
  return mt_next(r->g);
}
static const double MT_MAX = 4294967295.0;

/* ---------------------------------------------------------------- context */
struct po_ctx {
  int n_bead, n_mol, n_type;
  double* x;   /* current xyz, unwrapped */
  double* t;   /* trial xyz */
  double* q;
  int* type;
  int* mol_start; /* n_mol+1 */
  char sym[MAXT][16];
  /* run.in: simulation.cc:30-50 */
  double box[3];
  int npbc;
  double beta, move_size;
  int calc_chem_pot, phantom, coion, grafted, grafted_counterion;
  double move_prob[5];
  /* force_field.cc:65-103 */
  int use_pair, use_ewald, use_bond, use_rigid, use_angle, use_dihed, use_ext,
      use_gc;
  double rigid;
  double lj_cut, lj_sig[MAXT], lj_eps[MAXT];
  double lB, dielectric, alpha;
  int dipole;
  double ebox[3], evol, real_cut, kc2;
  int real_cell[3], kcell[3];
  int n_k;
  double *kv, *kw, *sk; /* kv: n_k*3, kw: e^{-k2/4a}/k2, sk: n_k*2 */
  double kpref;         /* lB/(kPi V) * 4 kPi^2 */
  double k_bond, r0;
  double wall_cut, wall_sig[MAXT], wall_eps[MAXT];
  /* pair 0 TruncatedLJ, 1 HardSphere; external 0 TruncatedLJWall, 1
   * HardWall, 2 WellWall: radii per type, the well's width and depth */
  int pair_kind, ext_kind;
  double hs_rad[MAXT], wall_rad[MAXT], well_width, well_depth;
  int graft[MAXT]; /* 0 none, 1 "L", 2 "R" */
  /* wall-force pressure of slit systems (pressure.cc:400-488): the number of
   * evaluations and the accumulators p_tensor[0..11] */
  double vp_z, p_tensor[12];
  /* running totals (force_field.cc:1201-1219) */
  double e_pair, e_ewald, e_bond, e_ext, dipl_cur;
  double* bond_mol;
  /* counts (simulation.cc:1066-1094) */
  int n_chain, n_cion, n_aion, n_nion;
  /* grand-canonical species (force_field.cc:96-103) */
  double chem_pot, debroglie, gc_bead_charge;
  int gc_freq, gc_chain_len, cbmc_trials, gc_type;
  /* gasdev's cached second deviate (misc.cc:112-113 keeps it in statics) */
  int gd_iset;
  double gd_gset;
  mt_t g;
};

int po_n_bead(const po_ctx* c) { return c->n_bead; }
int po_n_mol(const po_ctx* c) { return c->n_mol; }
int po_n_kvec(const po_ctx* c) { return c->n_k; }

/* ------------------------------------------------------------- tokenizer */
typedef struct {
  char* buf;
  char* p;
} tok_t;

static int tok_open(tok_t* t, const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  t->buf = (char*)malloc((size_t)n + 1);
  size_t got = fread(t->buf, 1, (size_t)n, f);
  t->buf[got] = 0;
  fclose(f);
  t->p = t->buf;
  return 0;
}

static const char* tok_next(tok_t* t) {
  while (*t->p && (*t->p == ' ' || *t->p == '\t' || *t->p == '\n' || *t->p == '\r'))
    t->p++;
  if (!*t->p) return NULL;
  char* s = t->p;
  while (*t->p && !(*t->p == ' ' || *t->p == '\t' || *t->p == '\n' || *t->p == '\r'))
    t->p++;
  if (*t->p) *t->p++ = 0;
  return s;
}

typedef struct {
  tok_t* t;
  char* err;
  int cap;
  int bad;
} rd_t;

static void rd_fail(rd_t* r, const char* fmt, ...) {
  if (r->bad) return;
  r->bad = 1;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(r->err, (size_t)r->cap, fmt, ap);
  va_end(ap);
}

/* `flag value` item: skips the flag, returns the value token. */
static const char* rd_item(rd_t* r, const char* what) {
  if (r->bad) return "0";
  const char* f = tok_next(r->t);
  const char* v = f ? tok_next(r->t) : NULL;
  if (!v) {
    rd_fail(r, "run.in ended while reading %s", what);
    return "0";
  }
  return v;
}
static double rd_d(rd_t* r, const char* w) { return atof(rd_item(r, w)); }
static int rd_i(rd_t* r, const char* w) { return atoi(rd_item(r, w)); }

static int type_of(po_ctx* c, const char* s) {
  for (int i = 0; i < c->n_type; i++)
    if (!strcmp(c->sym[i], s)) return i;
  if (c->n_type >= MAXT) return -1;
  snprintf(c->sym[c->n_type], 16, "%s", s);
  c->lj_sig[c->n_type] = c->lj_eps[c->n_type] = 0.0;
  c->wall_sig[c->n_type] = c->wall_eps[c->n_type] = 0.0;
  c->hs_rad[c->n_type] = c->wall_rad[c->n_type] = 0.0;
  c->graft[c->n_type] = !strcmp(s, "L") ? 1 : (!strcmp(s, "R") ? 2 : 0);
  return c->n_type++;
}

/* {symbol sigma epsilon}... end  (potential_truncated_lj.cc:31-45,
 * potential_truncated_lj_wall.cc:29-43). Symbols absent from the table keep
 * sigma = epsilon = 0, as std::map::operator[] gives the reference. */
static void rd_table(rd_t* r, po_ctx* c, double* sig, double* eps) {
  for (int guard = 0; guard < 100000 && !r->bad; guard++) {
    const char* s = rd_item(r, "bead type symbol");
    if (r->bad) return;
    if (!strcmp(s, "end")) return;
    char name[16];
    snprintf(name, 16, "%s", s);
    double sg = rd_d(r, "sigma"), ep = rd_d(r, "epsilon");
    int ti = type_of(c, name);
    if (ti < 0) {
      rd_fail(r, "too many bead types");
      return;
    }
    sig[ti] = sg;
    eps[ti] = ep;
  }
}

/* {symbol radius}... end (potential_hard_sphere.cc:20-36,
 * potential_hard_wall.cc:15-33, potential_well_wall.cc:24-37); absent
 * symbols keep radius 0 as std::map::operator[] gives the reference. */
static void rd_radii(rd_t* r, po_ctx* c, double* rad) {
  for (int guard = 0; guard < 100000 && !r->bad; guard++) {
    const char* s = rd_item(r, "bead type symbol");
    if (r->bad) return;
    if (!strcmp(s, "end")) return;
    char name[16];
    snprintf(name, 16, "%s", s);
    double v = rd_d(r, "radius");
    int ti = type_of(c, name);
    if (ti < 0) {
      rd_fail(r, "too many bead types");
      return;
    }
    rad[ti] = v;
  }
}

static char* join_path(const char* dir, const char* name) {
  size_t n = strlen(dir) + strlen(name) + 2;
  char* p = (char*)malloc(n);
  if (name[0] == '/')
    snprintf(p, n, "%s", name);
  else
    snprintf(p, n, "%s/%s", dir, name);
  return p;
}

/* ------------------------------------------------------------ geometry */
/* Bead::BBDist on two coordinate triples (bead.cc:162-176). */
static double bbdist(const double* a, const double* b, const double* box,
                     int npbc) {
  double dist = 0;
  for (int i = 0; i < 3; i++) {
    double di = a[i] - b[i];
    if (i < npbc) {
      di -= box[i] * round(di / box[i]);
      if (fabs(di) > 0.5 * box[i]) di = box[i] - fabs(di);
    }
    dist += (di * di);
  }
  return sqrt(dist);
}

/* PotentialTruncatedLJ::PairEnergy (potential_truncated_lj.cc:49-85). */
static double lj_pair(const po_ctx* c, const double* a, int ta, const double* b,
                      int tb) {
  double energy = 0;
  double r = bbdist(a, b, c->box, c->npbc);
  if (c->pair_kind == 1) /* PotentialHardSphere::PairEnergy (potential_hard_sphere.cc:38-49) */
    return r <= c->hs_rad[ta] + c->hs_rad[tb] ? K_VERY_LARGE : 0;
  double sigma = (c->lj_sig[ta] + c->lj_sig[tb]) / 2;
  double epsilon = sqrt((c->lj_eps[ta] * c->lj_eps[tb]));
  if (r <= 0) return K_VERY_LARGE;
  if (c->lj_cut < 0) {
    double r6_ref = pow((1.0 / K216), 6);
    double energy_ref = 4 * epsilon * (r6_ref * r6_ref - r6_ref);
    if (r < K216 * sigma) {
      double r6 = pow((sigma / r), 6);
      energy = 4 * epsilon * (r6 * r6 - r6) - energy_ref;
    }
  } else if (r < c->lj_cut) {
    double r6_ref = pow((sigma / c->lj_cut), 6);
    double energy_ref = 4 * epsilon * (r6_ref * r6_ref - r6_ref);
    double r6 = pow((sigma / r), 6);
    energy = 4 * epsilon * (r6 * r6 - r6) - energy_ref;
  }
  return energy;
}

/* PotentialEwaldCoul::PairEnergyReal (potential_ewald_coul.cc:134-164) with
 * GetDistVector (misc.cc:43-56) on the Ewald box. */
static double ew_real_pair(const po_ctx* c, const double* a, double qa,
                           const double* b, double qb) {
  double energy = 0;
  if (qa * qb == 0) return energy;
  double dist[3];
  for (int i = 0; i < 3; i++) {
    double di = b[i] - a[i];
    if (i < c->npbc) di -= c->ebox[i] * round(di / c->ebox[i]);
    dist[i] = di;
  }
  double prefactor = c->lB * qa * qb;
  for (int i = -c->real_cell[0]; i <= c->real_cell[0]; i++)
    for (int j = -c->real_cell[1]; j <= c->real_cell[1]; j++)
      for (int k = -c->real_cell[2]; k <= c->real_cell[2]; k++) {
        double rv0 = dist[0] + i * c->ebox[0];
        double rv1 = dist[1] + j * c->ebox[1];
        double rv2 = dist[2] + k * c->ebox[2];
        double r = sqrt(rv0 * rv0 + rv1 * rv1 + rv2 * rv2);
        if (r > 0 && r <= c->real_cut)
          energy += prefactor * erfc(sqrt(c->alpha) * r) / r;
      }
  return energy;
}

/* SelfEnergy (potential_ewald_coul.cc:253-257). */
static double ew_self(const po_ctx* c, double q) {
  return -c->lB * sqrt(c->alpha / K_PI) * q * q;
}

/* DipoleE on current z (potential_ewald_coul.cc:415-428). */
static double ew_dipole(const po_ctx* c) {
  double mz = 0;
  for (int i = 0; i < c->n_bead; i++) mz += c->q[i] * c->x[3 * i + 2];
  return c->lB * 2 * K_PI / (c->evol / 1.0) * mz * mz;
}

/* PotentialSpring::MoleculeEnergy (potential_spring.cc:22-48) on coords p. */
static double bond_mol_energy(const po_ctx* c, int m, const double* p) {
  double e = 0;
  for (int i = c->mol_start[m]; i < c->mol_start[m + 1] - 1; i++) {
    double r = bbdist(p + 3 * i, p + 3 * (i + 1), c->box, 0);
    e += 0.5 * c->k_bond * (r - c->r0) * (r - c->r0);
  }
  return e;
}

/* PotentialTruncatedLJWall::BeadEnergy (potential_truncated_lj_wall.cc:46-134). */
static double wall_energy(const po_ctx* c, double z, int ty) {
  double energy = 0;
  if (c->ext_kind == 1) { /* PotentialHardWall::BeadEnergy (potential_hard_wall.cc:36-47) */
    const double rad = c->wall_rad[ty];
    return (z <= rad || z + rad >= c->box[2]) ? K_VERY_LARGE : 0;
  }
  if (c->ext_kind == 2) { /* PotentialWellWall::BeadEnergy (potential_well_wall.cc:41-55) */
    const double rad = c->wall_rad[ty];
    if (z <= rad || z >= c->box[2] - rad) return K_VERY_LARGE;
    if (z < c->well_width || z > c->box[2] - c->well_width) return c->well_depth;
    return 0;
  }
  double sigma = c->wall_sig[ty], epsilon = c->wall_eps[ty];
  double R0 = 3 * K213 * sigma, K = 1;
  double lz = c->box[2];
  int g = c->graft[ty];
  if (epsilon == 0) return 0;
  if (z <= 0 || z >= lz) return K_VERY_LARGE;
  if (c->wall_cut < 0 && g == 0) {
    double r3_ref = pow((1.0 / K213), 3);
    double energy_ref = 2.59807621135 * epsilon * (r3_ref * r3_ref - r3_ref);
    if (z < K213 * sigma) {
      double r3 = pow((sigma / z), 3);
      energy += 2.59807621135 * epsilon * (r3 * r3 - r3) - energy_ref;
    }
    if (lz - z < K213 * sigma) {
      double r3 = pow((sigma / (lz - z)), 3);
      energy += 2.59807621135 * epsilon * (r3 * r3 - r3) - energy_ref;
    }
  } else if (g == 1) {
    double r3 = pow((sigma / z), 3);
    energy += 2.59807621135 * epsilon * (r3 * r3 - r3);
    energy += -0.5 * K * R0 * R0 * log(1 - pow(z / R0, 2));
    if (lz - z < K213 * sigma) {
      r3 = pow((sigma / (lz - z)), 3);
      energy += 2.59807621135 * epsilon * (r3 * r3 - r3);
    } else {
      r3 = pow((1.0 / K213), 3);
      energy += 2.59807621135 * epsilon * (r3 * r3 - r3);
    }
  } else if (g == 2) {
    double r3 = pow((sigma / (lz - z)), 3);
    energy += 2.59807621135 * epsilon * (r3 * r3 - r3);
    energy += -0.5 * K * R0 * R0 * log(1 - pow((lz - z) / R0, 2));
    if (z < K213 * sigma) {
      r3 = pow((sigma / z), 3);
      energy += 2.59807621135 * epsilon * (r3 * r3 - r3);
    } else {
      r3 = pow((1.0 / K213), 3);
      energy += 2.59807621135 * epsilon * (r3 * r3 - r3);
    }
  } else {
    double r3_ref = pow((1.0 / c->wall_cut), 3);
    double energy_ref = 2.59807621135 * epsilon * (r3_ref * r3_ref - r3_ref);
    if (z < c->wall_cut) {
      double r3 = pow((sigma / z), 3);
      energy += 2.59807621135 * epsilon * (r3 * r3 - r3) - energy_ref;
    }
    if (lz - z < c->wall_cut) {
      double r3 = pow((sigma / (lz - z)), 3);
      energy += 2.59807621135 * epsilon * (r3 * r3 - r3) - energy_ref;
    }
  }
  return energy;
}

/* Structure factor contribution of one bead: q e^{i k.r} for every k in the
 * half space, positions wrapped into the primary cell on periodic axes. */
static void sk_add(const po_ctx* c, const double* p, double q, double sign,
                   double* acc) {
  double w[3];
  for (int a = 0; a < 3; a++) {
    w[a] = p[a];
    if (a < c->npbc) w[a] -= c->ebox[a] * floor(p[a] / c->ebox[a]);
  }
  for (int k = 0; k < c->n_k; k++) {
    double ph = c->kv[3 * k] * w[0] + c->kv[3 * k + 1] * w[1] + c->kv[3 * k + 2] * w[2];
    acc[2 * k] += sign * q * cos(ph);
    acc[2 * k + 1] += sign * q * sin(ph);
  }
}

static double sk_energy(const po_ctx* c, const double* s) {
  double e = 0;
  for (int k = 0; k < c->n_k; k++)
    e += c->kw[k] * (s[2 * k] * s[2 * k] + s[2 * k + 1] * s[2 * k + 1]);
  return c->kpref * e;
}

/* ----------------------------------------------------------- Ewald setup */
/* PotentialEwaldCoul::ReadParameters (potential_ewald_coul.cc:38-115), with
 * optional overrides from the trailing extension block. */
static void ewald_setup(po_ctx* c, double rc_over, int kmax_over, double kc2_over,
                        int have_kc2) {
  for (int i = 0; i < 3; i++) c->ebox[i] = c->box[i];
  if (c->dipole) {
    double min_padding = 150;
    if (c->ebox[2] * K_DI_CORRECTION > min_padding)
      c->ebox[2] = c->ebox[2] * K_DI_CORRECTION;
    else
      c->ebox[2] += min_padding;
  }
  c->evol = c->ebox[0] * c->ebox[1] * c->ebox[2];
  c->real_cut = 1;
  while (0.5 * c->lB * 1 * 1 * erfc(sqrt(c->alpha) * c->real_cut) / c->real_cut >
         K_EWALD_CUTOFF)
    c->real_cut += 1;
  if (rc_over > 0) c->real_cut = rc_over;
  for (int i = 0; i < 3; i++) c->real_cell[i] = (int)ceil(c->real_cut / c->ebox[i]);
  c->kc2 = c->alpha;
  double min_box_vol = pow(c->ebox[0], 3);
  while (c->lB * 1 * 1 / (2 * K_PI * min_box_vol) * (4 * K_PI * K_PI) *
             exp(-c->kc2 / (4 * c->alpha)) / c->kc2 >
         K_EWALD_CUTOFF)
    c->kc2 += c->alpha;
  for (int i = 0; i < 3; i++)
    c->kcell[i] = (int)ceil(sqrt(c->kc2) * c->ebox[i] / (2 * K_PI));
  if (kmax_over > 0) {
    for (int i = 0; i < 3; i++) c->kcell[i] = kmax_over;
    if (!have_kc2) c->kc2 = INFINITY;
  }
  if (have_kc2) c->kc2 = kc2_over > 0 ? kc2_over : INFINITY;
  int cap = (2 * c->kcell[0] + 1) * (2 * c->kcell[1] + 1) * (2 * c->kcell[2] + 1);
  c->kv = (double*)malloc(sizeof(double) * 3 * (size_t)cap);
  c->kw = (double*)malloc(sizeof(double) * (size_t)cap);
  c->n_k = 0;
  for (int lx = -c->kcell[0]; lx <= c->kcell[0]; lx++)
    for (int ly = -c->kcell[1]; ly <= c->kcell[1]; ly++)
      for (int lz = -c->kcell[2]; lz <= c->kcell[2]; lz++) {
        int half = lx > 0 || (lx == 0 && ly > 0) || (lx == 0 && ly == 0 && lz > 0);
        if (!half) continue;
        double kx = lx * 2 * K_PI / c->ebox[0];
        double ky = ly * 2 * K_PI / c->ebox[1];
        double kz = lz * 2 * K_PI / c->ebox[2];
        double k2 = kx * kx + ky * ky + kz * kz;
        if (!(k2 > 0 && k2 <= c->kc2)) continue;
        c->kv[3 * c->n_k] = kx;
        c->kv[3 * c->n_k + 1] = ky;
        c->kv[3 * c->n_k + 2] = kz;
        c->kw[c->n_k] = exp(-k2 / (4 * c->alpha)) / k2;
        c->n_k++;
      }
  c->kpref = c->lB / (K_PI * c->evol) * (4 * K_PI * K_PI);
  c->sk = (double*)calloc((size_t)2 * (c->n_k > 0 ? c->n_k : 1), sizeof(double));
}

void po_ewald_info(const po_ctx* c, double* out) {
  out[0] = c->real_cut;
  out[1] = c->kc2;
  for (int i = 0; i < 3; i++) out[2 + i] = c->real_cell[i];
  for (int i = 0; i < 3; i++) out[5 + i] = c->kcell[i];
  for (int i = 0; i < 3; i++) out[8 + i] = c->ebox[i];
  out[11] = c->alpha;
  out[12] = c->lB;
  out[13] = c->evol;
  out[14] = c->dipole;
}

/* simulation.cc:1066-1094 */
static void update_counts(po_ctx* c) {
  c->n_chain = c->n_cion = c->n_aion = c->n_nion = 0;
  for (int m = c->phantom; m < c->n_mol; m++) {
    int sz = c->mol_start[m + 1] - c->mol_start[m];
    double q0 = c->q[c->mol_start[m]];
    if (sz > 1)
      c->n_chain++;
    else if (q0 > 0)
      c->n_cion++;
    else if (q0 < 0)
      c->n_aion++;
    else
      c->n_nion++;
  }
  c->n_chain -= c->grafted;
}

/* ------------------------------------------------------------- creation */
static int g_skip_pair_totals = 0;

void po_set_fast_init(int on) { g_skip_pair_totals = on; }

po_ctx* po_create(const char* dir, const char* runin, uint32_t seed, char* err,
                  int cap) {
  po_ctx* c = (po_ctx*)calloc(1, sizeof(po_ctx));
  tok_t tr, tt, tc;
  memset(&tr, 0, sizeof(tr));
  memset(&tt, 0, sizeof(tt));
  memset(&tc, 0, sizeof(tc));
  rd_t r = {&tr, err, cap, 0};
  char* p = join_path(dir, runin);
  if (tok_open(&tr, p)) {
    snprintf(err, (size_t)cap, "cannot open %s", p);
    free(p);
    free(c);
    return NULL;
  }
  free(p);
  char crd[512], top[512];
  snprintf(crd, sizeof crd, "%s", rd_item(&r, "crd name"));
  snprintf(top, sizeof top, "%s", rd_item(&r, "top name"));
  rd_item(&r, "run name");
  rd_item(&r, "steps");
  rd_item(&r, "steps_eq");
  rd_item(&r, "sample_freq");
  rd_item(&r, "stat_out_freq");
  rd_item(&r, "traj_out_freq");
  c->npbc = rd_i(&r, "npbc");
  c->beta = rd_d(&r, "beta");
  c->move_size = rd_d(&r, "move_size");
  c->calc_chem_pot = rd_i(&r, "calc_chem_pot");
  c->phantom = rd_i(&r, "phantom");
  c->coion = rd_i(&r, "coion");
  c->grafted = rd_i(&r, "grafted");
  c->grafted_counterion = rd_i(&r, "grafted_counterion");
  for (int i = 0; i < 5; i++) c->move_prob[i] = rd_d(&r, "move_prob");
  rd_item(&r, "vp_el_res");
  rd_item(&r, "vp_bead_size");
  c->use_pair = rd_i(&r, "use_pair");
  c->use_ewald = rd_i(&r, "use_ewald");
  c->use_bond = rd_i(&r, "use_bond");
  c->use_rigid = rd_i(&r, "use_bond_rigid");
  c->use_angle = rd_i(&r, "use_angle");
  c->use_dihed = rd_i(&r, "use_dihed");
  c->use_ext = rd_i(&r, "use_ext");
  c->use_gc = rd_i(&r, "use_gc");
  char gc_sym[64] = "";
  if (c->use_gc) {
    c->chem_pot = rd_d(&r, "chemical potential");
    c->debroglie = rd_d(&r, "de Broglie prefactor");
    c->gc_freq = rd_i(&r, "GC frequency");
    c->gc_chain_len = rd_i(&r, "GC chain length");
    c->gc_bead_charge = rd_d(&r, "GC bead charge");
    snprintf(gc_sym, sizeof gc_sym, "%s", rd_item(&r, "GC bead symbol"));
    c->cbmc_trials = rd_i(&r, "CBMC trials");
  }
  c->rigid = -1;
  if (c->use_pair) {
    const char* nm = rd_item(&r, "pair potential");
    if (!strcmp(nm, "HardSphere")) {
      c->pair_kind = 1;
      rd_radii(&r, c, c->hs_rad);
    } else {
      if (strcmp(nm, "TruncatedLJ")) rd_fail(&r, "unsupported pair potential %s", nm);
      c->lj_cut = rd_d(&r, "LJ cutoff");
      rd_table(&r, c, c->lj_sig, c->lj_eps);
    }
  }
  if (c->use_ewald) {
    const char* nm = rd_item(&r, "Ewald potential");
    if (strcmp(nm, "Coul")) rd_fail(&r, "unsupported Ewald potential %s", nm);
    c->lB = rd_d(&r, "lB");
    c->dielectric = rd_d(&r, "dielectric");
    c->alpha = rd_d(&r, "alpha");
    c->dipole = rd_i(&r, "dipole correction");
  }
  if (c->use_bond) {
    const char* nm = rd_item(&r, "bond potential");
    if (strcmp(nm, "Spring")) rd_fail(&r, "unsupported bond potential %s", nm);
    c->k_bond = rd_d(&r, "k");
    c->r0 = rd_d(&r, "r0");
  }
  if (c->use_rigid) c->rigid = rd_d(&r, "rigid bond");
  if (c->use_ext) {
    const char* nm = rd_item(&r, "external potential");
    if (!strcmp(nm, "HardWall")) {
      c->ext_kind = 1;
      rd_radii(&r, c, c->wall_rad);
    } else if (!strcmp(nm, "WellWall")) {
      c->ext_kind = 2;
      c->well_width = rd_d(&r, "well width");
      c->well_depth = rd_d(&r, "well depth");
      rd_radii(&r, c, c->wall_rad);
    } else {
      if (strcmp(nm, "TruncatedLJWall")) rd_fail(&r, "unsupported external potential %s", nm);
      c->wall_cut = rd_d(&r, "wall cutoff");
      rd_item(&r, "wall sigma");
      rd_item(&r, "wall epsilon");
      rd_table(&r, c, c->wall_sig, c->wall_eps);
    }
  }
  /* Trailing extension block (never read by the reference). */
  double rc_over = -1, kc2_over = -1;
  int kmax_over = -1, have_kc2 = 0;
  for (;;) {
    const char* key = tok_next(&tr);
    const char* val = key ? tok_next(&tr) : NULL;
    if (!val) break;
    if (!strcmp(key, "plum_ewald_real_cutoff")) rc_over = atof(val);
    if (!strcmp(key, "plum_ewald_kmax")) kmax_over = atoi(val);
    if (!strcmp(key, "plum_ewald_kcut2")) {
      kc2_over = atof(val);
      have_kc2 = 1;
    }
  }
  if (r.bad) goto fail;
  c->gc_type = c->use_gc ? type_of(c, gc_sym) : -1;
  /* top file: simulation.cc:610-646 */
  p = join_path(dir, top);
  if (tok_open(&tt, p)) {
    snprintf(err, (size_t)cap, "cannot open %s", p);
    free(p);
    goto fail;
  }
  free(p);
  {
    rd_t rt = {&tt, err, cap, 0};
    rd_item(&rt, "n_bead");
    c->n_mol = rd_i(&rt, "n_mol");
    for (int i = 0; i < 3; i++) c->box[i] = rd_d(&rt, "box");
    if (rt.bad || c->n_mol <= 0) {
      if (!rt.bad) snprintf(err, (size_t)cap, "bad molecule count");
      goto fail;
    }
  }
  /* crd file: simulation.cc:582-608 */
  p = join_path(dir, crd);
  {
    FILE* f = fopen(p, "r");
    free(p);
    if (!f) {
      snprintf(err, (size_t)cap, "cannot open coordinate file");
      goto fail;
    }
    char line[1024];
    if (!fgets(line, sizeof line, f) || !fgets(line, sizeof line, f)) {
      fclose(f);
      snprintf(err, (size_t)cap, "coordinate file too short");
      goto fail;
    }
    int capb = 1024, nb = 0;
    int* mol = (int*)malloc(sizeof(int) * capb);
    double* xyz = (double*)malloc(sizeof(double) * 3 * capb);
    double* qq = (double*)malloc(sizeof(double) * capb);
    int* ty = (int*)malloc(sizeof(int) * capb);
    int mid;
    char s[64];
    double x, y, z, q;
    while (fscanf(f, "%d %63s %lf %lf %lf %lf", &mid, s, &x, &y, &z, &q) == 6) {
      if (mid < 0 || mid >= c->n_mol) {
        snprintf(err, (size_t)cap, "Molecule ID %d is out of bounds", mid);
        fclose(f);
        free(mol), free(xyz), free(qq), free(ty);
        goto fail;
      }
      if (nb == capb) {
        capb *= 2;
        mol = (int*)realloc(mol, sizeof(int) * capb);
        xyz = (double*)realloc(xyz, sizeof(double) * 3 * capb);
        qq = (double*)realloc(qq, sizeof(double) * capb);
        ty = (int*)realloc(ty, sizeof(int) * capb);
      }
      mol[nb] = mid;
      xyz[3 * nb] = x, xyz[3 * nb + 1] = y, xyz[3 * nb + 2] = z;
      qq[nb] = q;
      ty[nb] = type_of(c, s);
      nb++;
    }
    fclose(f);
    /* Molecules are stored in molecule order; beads keep file order within a
     * molecule (Molecule::AddBead, molecule.cc:47-52). */
    c->n_bead = nb;
    c->mol_start = (int*)calloc((size_t)c->n_mol + 1, sizeof(int));
    for (int i = 0; i < nb; i++) c->mol_start[mol[i] + 1]++;
    for (int m = 0; m < c->n_mol; m++) {
      if (c->mol_start[m + 1] == 0) {
        snprintf(err, (size_t)cap, "molecule %d has no beads", m);
        free(mol), free(xyz), free(qq), free(ty);
        goto fail;
      }
      c->mol_start[m + 1] += c->mol_start[m];
    }
    int* fill = (int*)calloc((size_t)c->n_mol, sizeof(int));
    c->x = (double*)malloc(sizeof(double) * 3 * nb);
    c->t = (double*)malloc(sizeof(double) * 3 * nb);
    c->q = (double*)malloc(sizeof(double) * nb);
    c->type = (int*)malloc(sizeof(int) * nb);
    for (int i = 0; i < nb; i++) {
      int k = c->mol_start[mol[i]] + fill[mol[i]]++;
      memcpy(c->x + 3 * k, xyz + 3 * i, 3 * sizeof(double));
      c->q[k] = qq[i];
      c->type[k] = ty[i];
    }
    memcpy(c->t, c->x, sizeof(double) * 3 * nb);
    free(fill), free(mol), free(xyz), free(qq), free(ty);
  }
  if (c->use_ewald) ewald_setup(c, rc_over, kmax_over, kc2_over, have_kc2);
  c->bond_mol = (double*)calloc((size_t)c->n_mol, sizeof(double));
  update_counts(c);
  mt_seed(&c->g, seed);
  {
    double e[8];
    po_total_energy(c, e);
  }
  free(tr.buf), free(tt.buf), free(tc.buf);
  return c;
fail:
  free(tr.buf), free(tt.buf), free(tc.buf);
  po_destroy(c);
  return NULL;
}

void po_destroy(po_ctx* c) {
  if (!c) return;
  free(c->x), free(c->t), free(c->q), free(c->type), free(c->mol_start);
  free(c->kv), free(c->kw), free(c->sk), free(c->bond_mol);
  free(c);
}

static int mol_of(const po_ctx* c, int bead) {
  int lo = 0, hi = c->n_mol - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) / 2;
    if (c->mol_start[mid] <= bead)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

/* ------------------------------------------------------- total energy */
/* ForceField::InitializeEnergy (force_field.cc:365-381) through the
 * potentials' EnergyInitialization; pairs in the reference's loop order
 * (intramolecular first, then molecule pairs), potential_pair.cc:55-100. */
void po_total_energy(po_ctx* c, double* out) {
  double ep = 0, er = 0, ek = 0, es = 0, ed = 0, eb = 0, ee = 0;
  const int skip = g_skip_pair_totals;
  if (c->use_pair && !skip) {
    for (int m = 0; m < c->n_mol; m++)
      for (int j = c->mol_start[m]; j < c->mol_start[m + 1] - 1; j++)
        for (int k = j + 1; k < c->mol_start[m + 1]; k++)
          if (!(c->pair_kind == 1 && k == j + 1))  /* hard spheres skip bonded neighbours */
            ep += lj_pair(c, c->x + 3 * j, c->type[j], c->x + 3 * k, c->type[k]);
    for (int m = 0; m < c->n_mol - 1; m++)
      for (int i = c->mol_start[m]; i < c->mol_start[m + 1]; i++)
        for (int j = c->mol_start[m + 1]; j < c->n_bead; j++)
          ep += lj_pair(c, c->x + 3 * i, c->type[i], c->x + 3 * j, c->type[j]);
  }
  if (c->use_ewald) {
    for (int i = 0; i < c->n_bead && !skip; i++) {
      er += 0.5 * ew_real_pair(c, c->x + 3 * i, c->q[i], c->x + 3 * i, c->q[i]);
      for (int j = i + 1; j < c->n_bead; j++)
        er += ew_real_pair(c, c->x + 3 * i, c->q[i], c->x + 3 * j, c->q[j]);
    }
    memset(c->sk, 0, sizeof(double) * 2 * (size_t)c->n_k);
    for (int i = 0; i < c->n_bead; i++) sk_add(c, c->x + 3 * i, c->q[i], 1.0, c->sk);
    ek = sk_energy(c, c->sk);
    for (int i = 0; i < c->n_bead; i++) es += ew_self(c, c->q[i]);
    if (c->dipole) ed = ew_dipole(c);
    c->dipl_cur = ed;
  }
  if (c->use_bond)
    for (int m = 0; m < c->n_mol; m++) {
      c->bond_mol[m] = bond_mol_energy(c, m, c->x);
      eb += c->bond_mol[m];
    }
  if (c->use_ext)
    for (int i = 0; i < c->n_bead; i++) ee += wall_energy(c, c->x[3 * i + 2], c->type[i]);
  c->e_pair = ep;
  c->e_ewald = er + ek + es + ed;
  c->e_bond = eb;
  c->e_ext = ee;
  if (out) {
    out[0] = ep, out[1] = c->e_ewald, out[2] = eb, out[3] = ee;
    out[4] = er, out[5] = ek, out[6] = es, out[7] = ed;
  }
}

void po_energies(const po_ctx* c, double* out) {
  out[0] = c->e_pair, out[1] = c->e_ewald, out[2] = c->e_bond, out[3] = c->e_ext;
}

/* ----------------------------------------------------- energy difference */
typedef struct {
  double de, pair, ewald, bond, ext, dip_trial, bond_trial;
  double* dsk;
} de_t;

/* ForceField::EnergyDifference (force_field.cc:407-434) for molecule m with
 * trial coordinates c->t and flags mv (indexed by bead). */
static void energy_difference(po_ctx* c, int m, const int* mv, de_t* d) {
  int b0 = c->mol_start[m], b1 = c->mol_start[m + 1];
  d->pair = d->ewald = d->bond = d->ext = 0;
  d->de = 0;
  if (c->use_pair) {
    double de = 0;
    /* potential_pair.cc:152-201 */
    for (int i = b0; i < b1 - 1; i++)
      for (int j = i + 1; j < b1; j++)
        if ((mv[i] || mv[j]) && !(c->pair_kind == 1 && j == i + 1))
          de += lj_pair(c, c->t + 3 * i, c->type[i], c->t + 3 * j, c->type[j]) -
                lj_pair(c, c->x + 3 * i, c->type[i], c->x + 3 * j, c->type[j]);
    for (int o = 0; o < c->n_mol; o++) {
      if (o == m) continue;
      for (int j = c->mol_start[o]; j < c->mol_start[o + 1]; j++)
        for (int k = b0; k < b1; k++)
          if (mv[k])
            de += lj_pair(c, c->t + 3 * k, c->type[k], c->x + 3 * j, c->type[j]) -
                  lj_pair(c, c->x + 3 * k, c->type[k], c->x + 3 * j, c->type[j]);
    }
    d->pair = de;
    d->de += de;
    if (d->de >= K_VERY_LARGE) return;
  }
  if (c->use_ext) {
    /* potential_external.cc:100-117 */
    double de = 0;
    for (int i = b0; i < b1; i++) {
      if (!mv[i]) continue;
      double en = wall_energy(c, c->t[3 * i + 2], c->type[i]);
      if (en >= K_VERY_LARGE) {
        de = K_VERY_LARGE;
        break;
      }
      de += en - wall_energy(c, c->x[3 * i + 2], c->type[i]);
    }
    d->ext = de;
    d->de += de;
    if (d->de >= K_VERY_LARGE) return;
  }
  if (c->use_ewald) {
    /* potential_ewald.cc:429-535: real space pairwise (the i == j terms cancel
     * exactly), reciprocal space through S(k), self energy unchanged, dipole
     * from the current z (the reference evaluates DipoleE before commit). */
    double de = 0;
    for (int i = b0; i < b1; i++)
      for (int j = i + 1; j < b1; j++)
        if (mv[i] || mv[j])
          de += ew_real_pair(c, c->t + 3 * i, c->q[i], c->t + 3 * j, c->q[j]) -
                ew_real_pair(c, c->x + 3 * i, c->q[i], c->x + 3 * j, c->q[j]);
    for (int o = 0; o < c->n_mol; o++) {
      if (o == m) continue;
      for (int j = c->mol_start[o]; j < c->mol_start[o + 1]; j++)
        for (int k = b0; k < b1; k++)
          if (mv[k])
            de += ew_real_pair(c, c->t + 3 * k, c->q[k], c->x + 3 * j, c->q[j]) -
                  ew_real_pair(c, c->x + 3 * k, c->q[k], c->x + 3 * j, c->q[j]);
    }
    memset(d->dsk, 0, sizeof(double) * 2 * (size_t)c->n_k);
    for (int i = b0; i < b1; i++)
      if (mv[i] && c->q[i] != 0) {
        sk_add(c, c->t + 3 * i, c->q[i], 1.0, d->dsk);
        sk_add(c, c->x + 3 * i, c->q[i], -1.0, d->dsk);
      }
    double ek = 0;
    for (int k = 0; k < c->n_k; k++) {
      double sr = c->sk[2 * k], si = c->sk[2 * k + 1];
      double nr = sr + d->dsk[2 * k], ni = si + d->dsk[2 * k + 1];
      ek += c->kw[k] * ((nr * nr + ni * ni) - (sr * sr + si * si));
    }
    de += c->kpref * ek;
    if (c->dipole) {
      d->dip_trial = ew_dipole(c);
      de += d->dip_trial - c->dipl_cur;
    }
    d->ewald = de;
    d->de += de;
  }
  if (c->use_bond) {
    /* potential_spring.cc:63-80 */
    if (b1 - b0 > 1) {
      d->bond_trial = bond_mol_energy(c, m, c->t);
      d->bond = d->bond_trial - c->bond_mol[m];
      d->de += d->bond;
    }
  }
}

static void finalize(po_ctx* c, int m, const int* mv, const de_t* d, int accept) {
  int b0 = c->mol_start[m], b1 = c->mol_start[m + 1];
  if (accept) {
    c->e_pair += d->pair;
    c->e_ext += d->ext;
    c->e_ewald += d->ewald;
    c->e_bond += d->bond;
    if (c->use_ewald) {
      for (int k = 0; k < 2 * c->n_k; k++) c->sk[k] += d->dsk[k];
      if (c->dipole) c->dipl_cur = d->dip_trial;
    }
    if (c->use_bond && b1 - b0 > 1) c->bond_mol[m] = d->bond_trial;
    memcpy(c->x + 3 * b0, c->t + 3 * b0, sizeof(double) * 3 * (size_t)(b1 - b0));
  } else {
    memcpy(c->t + 3 * b0, c->x + 3 * b0, sizeof(double) * 3 * (size_t)(b1 - b0));
  }
  (void)mv;
}

void po_delta_energy(po_ctx* c, int mol, const double* trial, const int* moved,
                     double* out) {
  int b0 = c->mol_start[mol], b1 = c->mol_start[mol + 1];
  int* mv = (int*)calloc((size_t)c->n_bead, sizeof(int));
  for (int i = b0; i < b1; i++) {
    memcpy(c->t + 3 * i, trial + 3 * (i - b0), 3 * sizeof(double));
    mv[i] = moved[i - b0];
  }
  de_t d;
  memset(&d, 0, sizeof d);
  d.dsk = (double*)calloc((size_t)2 * (c->n_k > 0 ? c->n_k : 1), sizeof(double));
  energy_difference(c, mol, mv, &d);
  out[0] = d.de, out[1] = d.pair, out[2] = d.ewald, out[3] = d.bond, out[4] = d.ext;
  finalize(c, mol, mv, &d, 0);
  free(d.dsk);
  free(mv);
}

/* ------------------------------------------------------------------ moves */
/* randSphere (misc.cc:95-109) */
static void rand_sphere(rng_t* r, double* vec) {
  double rand_square = 2, r1 = 0, r2 = 0;
  while (rand_square > 1) {
    r1 = 1 - 2 * ((double)rng_u32(r) / MT_MAX);
    r2 = 1 - 2 * ((double)rng_u32(r) / MT_MAX);
    rand_square = r1 * r1 + r2 * r2;
    if (r->overrun) return;
  }
  double ranh = 2 * sqrt(1 - rand_square);
  vec[0] = r1 * ranh;
  vec[1] = r2 * ranh;
  vec[2] = (1 - 2 * rand_square);
}

#define TX(i, d) c->t[3 * (i) + (d)]
#define CX(i, d) c->x[3 * (i) + (d)]

/* Molecule::BeadTranslate (molecule.cc:103-133) */
static void mv_bead(po_ctx* c, rng_t* r, int b0, int* mv) {
  double vec[3];
  rand_sphere(r, vec);
  double vec_len = sqrt(vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2]);
  if (vec_len > 0) vec_len = 3 * c->move_size / vec_len;
  mv[b0] = 1;
  for (int i = 0; i < 3; i++) TX(b0, i) = CX(b0, i) + vec_len * vec[i];
}

/* Molecule::COMTranslate (molecule.cc:135-151) */
static void mv_com(po_ctx* c, rng_t* r, int b0, int b1, int* mv) {
  double vec[3];
  for (int i = 0; i < 3; i++) vec[i] = 0.5 * c->move_size * (double)rng_u32(r) / MT_MAX;
  for (int i = 0; i < 3; i++)
    if (rng_u32(r) % 2 == 0) vec[i] = -vec[i];
  for (int i = b0; i < b1; i++) {
    for (int j = 0; j < 3; j++) TX(i, j) = CX(i, j) + vec[j];
    mv[i] = 1;
  }
}

/* Molecule::Pivot (molecule.cc:153-237) */
static void mv_pivot(po_ctx* c, rng_t* r, int b0, int b1, double eq, int vary,
                     int* mv) {
  int len = b1 - b0;
  int pivot = (int)floor(len * (double)rng_u32(r) / MT_MAX);
  if (pivot == len) pivot--;
  double s = c->move_size * (double)rng_u32(r) / MT_MAX;
  for (int i = pivot + 1; i < len; i++) {
    double vec[3];
    rand_sphere(r, vec);
    int bi = b0 + i, bp = b0 + i - 1;
    double x = TX(bi, 0) + s * vec[0];
    double y = TX(bi, 1) + s * vec[1];
    double z = TX(bi, 2) + s * vec[2];
    double dx = x - TX(bp, 0), dy = y - TX(bp, 1), dz = z - TX(bp, 2);
    double bl = eq;
    if (vary) bl += (eq / 5.0) * ((double)rng_u32(r) / MT_MAX - 0.5);
    double norm = bl / sqrt(dx * dx + dy * dy + dz * dz);
    double cx = norm * dx + TX(bp, 0), cy = norm * dy + TX(bp, 1),
           cz = norm * dz + TX(bp, 2);
    double mx = cx - TX(bi, 0), my = cy - TX(bi, 1), mz = cz - TX(bi, 2);
    for (int j = i; j < len; j++) {
      TX(b0 + j, 0) = TX(b0 + j, 0) + mx;
      TX(b0 + j, 1) = TX(b0 + j, 1) + my;
      TX(b0 + j, 2) = TX(b0 + j, 2) + mz;
    }
  }
  for (int i = pivot - 1; i >= 0; i--) {
    double vec[3];
    rand_sphere(r, vec);
    int bi = b0 + i, bp = b0 + i + 1;
    double x = TX(bi, 0) + s * vec[0];
    double y = TX(bi, 1) + s * vec[1];
    double z = TX(bi, 2) + s * vec[2];
    double dx = x - TX(bp, 0), dy = y - TX(bp, 1), dz = z - TX(bp, 2);
    double bl = eq;
    if (vary) bl += (eq / 5.0) * ((double)rng_u32(r) / MT_MAX - 0.5);
    double norm = bl / sqrt(dx * dx + dy * dy + dz * dz);
    double cx = norm * dx + TX(bp, 0), cy = norm * dy + TX(bp, 1),
           cz = norm * dz + TX(bp, 2);
    double mx = cx - TX(bi, 0), my = cy - TX(bi, 1), mz = cz - TX(bi, 2);
    for (int j = i; j >= 0; j--) {
      TX(b0 + j, 0) = TX(b0 + j, 0) + mx;
      TX(b0 + j, 1) = TX(b0 + j, 1) + my;
      TX(b0 + j, 2) = TX(b0 + j, 2) + mz;
    }
  }
  for (int i = b0; i < b1; i++) mv[i] = 1;
}

/* Molecule::Crankshaft (molecule.cc:239-265). The rotation is Rodrigues'
 * formula in the per-entry grouping of Eigen's AngleAxis::toRotationMatrix. */
static void mv_crank(po_ctx* c, rng_t* r, int b0, int b1, int* mv) {
  int len = b1 - b0;
  int first = (int)floor((len - 2) * (double)rng_u32(r) / MT_MAX);
  int last = (int)floor((len - first) * (double)rng_u32(r) / MT_MAX) + first;
  if (last > len - 1) last = len - 1; /* the reference reads past the chain here */
  double ax[3];
  for (int i = 0; i < 3; i++) ax[i] = CX(b0 + last, i) - CX(b0 + first, i);
  double z = ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2];
  if (z > 0) {
    double n = sqrt(z);
    for (int i = 0; i < 3; i++) ax[i] /= n;
  }
  double angle = c->move_size * ((double)rng_u32(r) / MT_MAX * 2 * M_PI_LIBM - M_PI_LIBM);
  double sn = sin(angle), cs = cos(angle);
  double sa[3] = {sn * ax[0], sn * ax[1], sn * ax[2]};
  double ca[3] = {(1.0 - cs) * ax[0], (1.0 - cs) * ax[1], (1.0 - cs) * ax[2]};
  double R[3][3];
  double tt = ca[0] * ax[1];
  R[0][1] = tt - sa[2];
  R[1][0] = tt + sa[2];
  tt = ca[0] * ax[2];
  R[0][2] = tt + sa[1];
  R[2][0] = tt - sa[1];
  tt = ca[1] * ax[2];
  R[1][2] = tt - sa[0];
  R[2][1] = tt + sa[0];
  for (int i = 0; i < 3; i++) R[i][i] = ca[i] * ax[i] + cs;
  for (int i = first + 1; i < last; i++) {
    int bi = b0 + i;
    mv[bi] = 1;
    double v[3];
    for (int k = 0; k < 3; k++) v[k] = CX(bi, k) - CX(b0 + first, k);
    for (int k = 0; k < 3; k++)
      TX(bi, k) = ((R[k][0] * v[0] + R[k][1] * v[1]) + R[k][2] * v[2]) + CX(b0 + first, k);
  }
}

/* Molecule::RandomReptation (molecule.cc:267-312) */
static void mv_rept(po_ctx* c, rng_t* r, int b0, int b1, double eq, int vary,
                    int* mv) {
  int len = b1 - b0;
  double bl = eq;
  if (vary) bl += (eq / 5.0) * ((double)rng_u32(r) / MT_MAX - 0.5);
  int dir = 1, begin = 0, end = len - 1;
  if (rng_u32(r) % 2 == 0) {
    dir = -1;
    begin = len - 1;
    end = 0;
  }
  for (int i = begin; i != end; i += dir)
    for (int j = 0; j < 3; j++) TX(b0 + i, j) = CX(b0 + i + dir, j);
  double vec[3];
  rand_sphere(r, vec);
  double vl = sqrt(vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2]);
  for (int i = 0; i < 3; i++) TX(b0 + end, i) = CX(b0 + end, i) + bl * vec[i] / vl;
  for (int i = b0; i < b1; i++) mv[i] = 1;
}

/* Simulation::TranslationalMove (simulation.cc:241-355). Returns the move
 * type attempted (-1 if none); *acc receives the decision. */
static int translational_move(po_ctx* c, rng_t* r, int* mv, de_t* d, int* acc) {
  *acc = 0;
  if (c->n_mol - c->phantom <= 0) return -1;
  int n_ch = c->grafted + c->n_chain;
  int n_io = c->n_cion + c->n_aion + c->n_nion;
  int chain_id = -1, ion_id = -1;
  int which_chain = (int)floor((double)rng_u32(r) / MT_MAX * n_ch);
  int which_ion = (int)floor((double)rng_u32(r) / MT_MAX * n_io);
  if (which_chain == n_ch) which_chain--;
  if (which_ion == n_io) which_ion--;
  int ccount = -1, icount = -1;
  for (int i = c->phantom; i < c->n_mol; i++) {
    if (c->mol_start[i + 1] - c->mol_start[i] > 1)
      ccount++;
    else
      icount++;
    if (ccount == which_chain) {
      chain_id = i;
      which_chain = -2;
    }
    if (icount == which_ion) {
      ion_id = i;
      which_ion = -2;
    }
  }
  int move_type = 0;
  double u = (double)rng_u32(r) / MT_MAX;
  double cur = c->move_prob[0];
  while (cur < u && move_type < K_NO_MOVE_TYPE - 1) {
    move_type++;
    cur += c->move_prob[move_type];
  }
  if (cur < u) move_type++;
  if (move_type >= K_NO_MOVE_TYPE) move_type = K_NO_MOVE_TYPE - 1;
  int mol = -1;
  if (move_type == 0 && n_io > 0) {
    mol = ion_id;
    mv_bead(c, r, c->mol_start[mol], mv);
  } else if (n_ch > 0) {
    mol = chain_id;
    double bl = 0;
    int vary = 0;
    if (c->use_rigid) bl = c->rigid;
    if (c->use_bond) {
      bl = c->r0;
      vary = 1;
    }
    int b0 = c->mol_start[mol], b1 = c->mol_start[mol + 1];
    switch (move_type) {
      case 1: mv_com(c, r, b0, b1, mv); break;
      case 2: mv_pivot(c, r, b0, b1, bl, vary, mv); break;
      case 3: mv_crank(c, r, b0, b1, mv); break;
      case 4: mv_rept(c, r, b0, b1, bl, vary, mv); break;
    }
  }
  if (!((move_type == 0 && n_io > 0) || (move_type > 0 && n_ch > 0))) return -1;
  if (r->overrun) return -1;
  energy_difference(c, mol, mv, d);
  int accept = 0;
  /* simulation.cc:327-332: no draw only when dE >= 1e8 (a NaN dE still draws) */
  if (!(d->de >= K_VERY_LARGE)) accept = ((double)rng_u32(r) / MT_MAX < exp(-c->beta * d->de));
  finalize(c, mol, mv, d, accept);
  for (int i = c->mol_start[mol]; i < c->mol_start[mol + 1]; i++) mv[i] = 0;
  *acc = accept;
  return move_type;
}

static int gc_move(po_ctx* c, rng_t* r, int* acc);

static long run_loop(po_ctx* c, rng_t* r, int n, int* move_type, int* accept,
                     int* draws, double* etot) {
  int mv_cap = c->n_bead;
  int* mv = (int*)calloc((size_t)mv_cap, sizeof(int));
  de_t d;
  memset(&d, 0, sizeof d);
  d.dsk = (double*)calloc((size_t)2 * (c->n_k > 0 ? c->n_k : 1), sizeof(double));
  for (int s = 0; s < n; s++) {
    long p0 = r->pos;
    /* simulation.cc:221-226: int rand_num = rand_gen(); GC when
     * rand_num % gc_freq == 0 (signed, as the reference's int) */
    const int32_t rand_num = (int32_t)rng_u32(r);
    int acc = 0, mt;
    if (c->use_gc && c->gc_freq > 0 && rand_num % c->gc_freq == 0) {
      mt = gc_move(c, r, &acc);
      if (c->n_bead > mv_cap) {
        mv_cap = c->n_bead;
        free(mv);
        mv = (int*)calloc((size_t)mv_cap, sizeof(int));
      }
    } else {
      mt = translational_move(c, r, mv, &d, &acc);
    }
    if (r->overrun) break;
    if (move_type) move_type[s] = mt;
    if (accept) accept[s] = acc;
    if (draws) draws[s] = (int)(r->pos - p0);
    if (etot) etot[s] = c->e_pair + c->e_ewald + c->e_bond + c->e_ext;
  }
  free(d.dsk);
  free(mv);
  return r->overrun ? -1 : r->pos;
}

int po_run(po_ctx* c, int n, int* move_type, int* accept, int* draws,
           double* etot) {
  rng_t r = {&c->g, NULL, 0, 0, 0};
  run_loop(c, &r, n, move_type, accept, draws, etot);
  return n;
}

long po_run_stream(po_ctx* c, int n, const uint32_t* stream, long n_stream,
                   int* move_type, int* accept, double* etot) {
  rng_t r = {NULL, stream, n_stream, 0, 0};
  return run_loop(c, &r, n, move_type, accept, NULL, etot);
}

/* ------------------------------------------------------ grand canonical */
/* gasdev (misc.cc:111-134): polar Box-Muller; the second deviate is cached
 * (the reference keeps it in function statics shared by the process; here
 * per context, as in a fresh process). */
static double gasdev(po_ctx* c, rng_t* r, double mean, double sd) {
  if (c->gd_iset == 0) {
    double v1, v2, rsq;
    do {
      v1 = 2.0 * ((double)rng_u32(r) / MT_MAX) - 1.0;
      v2 = 2.0 * ((double)rng_u32(r) / MT_MAX) - 1.0;
      rsq = v1 * v1 + v2 * v2;
    } while ((rsq >= 1.0 || rsq == 0.0) && !r->overrun);
    if (r->overrun) return mean;
    double fac = sqrt(-2.0 * log(rsq) / rsq);
    c->gd_gset = v1 * fac;
    c->gd_iset = 1;
    return v2 * fac * sd + mean;
  }
  c->gd_iset = 0;
  return c->gd_gset * sd + mean;
}

/* PotentialSpring::RandomBondLen (potential_spring.cc:50-61): a Gaussian
 * around r0 accepted with probability len^2 / (r0 + 3 sigma)^2. */
static double random_bond_len(po_ctx* c, rng_t* r) {
  const double sigma = sqrt(1 / (c->beta * c->k_bond));
  const double a = (c->r0 + 3 * sigma) * (c->r0 + 3 * sigma);
  double len = 0;
  int ready = 0;
  while (!ready && !r->overrun) {
    len = gasdev(c, r, c->r0, sigma);
    ready = ((double)rng_u32(r) / MT_MAX < (len * len / a));
  }
  return len;
}

/* ForceField::UpdateMolCounts (force_field.cc:1258-1277): its counts put
 * neutral single beads with the cations. */
static void ff_counts(const po_ctx* c, int* n_chain, int* n_cion, int* n_aion) {
  *n_chain = *n_cion = *n_aion = 0;
  for (int m = c->phantom; m < c->n_mol; m++) {
    if (c->mol_start[m + 1] - c->mol_start[m] > 1)
      (*n_chain)++;
    else if (c->q[c->mol_start[m]] >= 0)
      (*n_cion)++;
    else
      (*n_aion)++;
  }
  *n_chain -= c->grafted;
}

/* ForceField::CBMCFGenTrialBeads (cbmc.cc:161-212): each trial draws its
 * bond length, its direction and (charged species) its counterion's
 * position, then gets its Boltzmann weight; returns the weights' sum. */
static double gen_trials(po_ctx* c, rng_t* r, const double* end, int cl, const double* chain,
                         const double* chain_ci, int delete_id, double* tb1, double* tb2,
                         double* w) {
  const int charged = c->gc_bead_charge != 0;
  double Wi = 0;
  for (int i = 0; i < c->cbmc_trials; i++) {
    double bl = 0;
    if (c->use_bond)
      bl = random_bond_len(c, r);
    else if (c->use_rigid)
      bl = c->rigid;
    double v[3] = {0, 0, 0};
    rand_sphere(r, v);
    for (int j = 0; j < 3; j++) tb1[3 * i + j] = v[j] * bl + end[j];
    if (charged)
      for (int j = 0; j < 3; j++) tb2[3 * i + j] = (double)rng_u32(r) / MT_MAX * c->box[j];
    if (r->overrun) return 0;
    const double u = po_beads_energy(c, tb1 + 3 * i, charged ? tb2 + 3 * i : tb1 + 3 * i, cl,
                                     chain, chain_ci, delete_id);
    w[i] = exp(-c->beta * u);
    Wi += w[i];
  }
  return Wi;
}

/* spc1: molecules of the exchanged species; spc2: its counter-species
 * (cbmc.cc:265-275, 336-340, 407-411). */
static void gc_species(const po_ctx* c, int* spc1, int* spc2) {
  int nc, ncat, nan;
  ff_counts(c, &nc, &ncat, &nan);
  const double qb = c->gc_bead_charge;
  if (c->gc_chain_len > 1)
    *spc1 = nc;
  else if (qb >= 0)
    *spc1 = ncat - c->coion;
  else
    *spc1 = nan - c->coion;
  *spc2 = qb == 0 ? 0 : (qb > 0 ? nan : ncat);
}

/* ForceField::CBMCFChainInsertion (cbmc.cc:214-328); chain [2L][3] gets the
 * grown chain and (charged species) its counterions. */
static int chain_insertion(po_ctx* c, rng_t* r, double* chain) {
  const int L = c->gc_chain_len, T = c->cbmc_trials;
  const int charged = c->gc_bead_charge != 0;
  double weight = 1.0;
  const int i_index = charged ? L : 0, initial = charged ? 2 : 1;
  for (int i = 0; i < initial; i++)
    for (int j = 0; j < 3; j++) chain[3 * (i * L) + j] = (double)rng_u32(r) / MT_MAX * c->box[j];
  if (r->overrun) return 0;
  weight *= exp(-c->beta * po_beads_energy(c, chain, chain + 3 * i_index, 0, chain,
                                            chain + 3 * L, -1));
  if (weight <= 0) return 0;
  double* tb1 = (double*)malloc(sizeof(double) * 3 * (size_t)T);
  double* tb2 = (double*)malloc(sizeof(double) * 3 * (size_t)T);
  double* w = (double*)malloc(sizeof(double) * (size_t)T);
  int ok = 1;
  for (int i = 1; i < L && ok; i++) {
    const double Wi = gen_trials(c, r, chain + 3 * (i - 1), i, chain, chain + 3 * L, -1, tb1,
                                 tb2, w);
    weight *= Wi / T;
    if (r->overrun || weight <= 0) {
      ok = 0;
      break;
    }
    const double rn = (double)rng_u32(r) / MT_MAX * Wi;
    int cb = 0;
    double cum = w[0];
    while (cum < rn && cb < T - 1) cum += w[++cb];
    for (int j = 0; j < 3; j++) chain[3 * i + j] = tb1[3 * cb + j];
    if (charged)
      for (int j = 0; j < 3; j++) chain[3 * (i + L) + j] = tb2[3 * cb + j];
  }
  free(tb1);
  free(tb2);
  free(w);
  if (!ok || r->overrun) return 0;
  int spc1, spc2;
  gc_species(c, &spc1, &spc2);
  const int spc2_add = charged ? L : 0;
  double factorial = 1;
  for (int i = spc1 + 1; i <= spc1 + 1; i++) factorial *= i;
  for (int i = spc2 + 1; i <= spc2 + spc2_add; i++) factorial *= i;
  const double vol = c->box[0] * c->box[1] * c->box[2];
  double vol_over_lam = 1;
  vol_over_lam *= pow(vol / (c->debroglie / pow((double)L, 1.5)), 1);
  vol_over_lam *= pow(vol / (c->debroglie / pow(1.0, 1.5)), spc2_add);
  const double C = vol_over_lam * (1.0 / factorial);
  const double rn = (double)rng_u32(r) / MT_MAX;
  return rn < (exp(c->beta * c->chem_pot) * weight) * C;
}

/* ForceField::CalcChemicalPotentialF (cbmc.cc:444-531): Widom's test
 * insertion of the exchanged species grown by configurational bias,
 * averaged over n_ins insertions (mu_tot_ins = 50, force_field.cc:236) with
 * the reference's prefactor (its volume divided by 15.625, unlike the
 * insertion move's) and an overlap test by equality with 1e8. */
static double chem_pot_widom(po_ctx* c, rng_t* r, int n_ins) {
  const int L = c->gc_chain_len, T = c->cbmc_trials;
  const int charged = c->gc_bead_charge != 0;
  int spc1, spc2;
  gc_species(c, &spc1, &spc2);
  const int spc2_add = charged ? L : 0;
  double factorial = 1;
  for (int i = spc1 + 1; i <= spc1 + 1; i++) factorial *= i;
  for (int i = spc2 + 1; i <= spc2 + spc2_add; i++) factorial *= i;
  const double vol = c->box[0] * c->box[1] * c->box[2];
  double vol_over_lam = 1;
  vol_over_lam *= pow(vol / 15.625 / (c->debroglie / pow((double)L, 1.5)), 1);
  vol_over_lam *= pow(vol / 15.625 / (c->debroglie / pow(1.0, 1.5)), spc2_add);
  const double C = vol_over_lam * (1.0 / factorial);
  double* chain = (double*)calloc((size_t)6 * (L > 0 ? L : 1), sizeof(double));
  double* tb1 = (double*)malloc(sizeof(double) * 3 * (size_t)T);
  double* tb2 = (double*)malloc(sizeof(double) * 3 * (size_t)T);
  double* w = (double*)malloc(sizeof(double) * (size_t)T);
  double total = 0;
  for (int n = 0; n < n_ins && !r->overrun; n++) {
    double weight = 1.0;
    const int i_index = charged ? L : 0, initial = charged ? 2 : 1;
    for (int i = 0; i < initial; i++)
      for (int j = 0; j < 3; j++) chain[3 * (i * L) + j] = (double)rng_u32(r) / MT_MAX * c->box[j];
    const double dE = po_beads_energy(c, chain, chain + 3 * i_index, 0, chain, chain + 3 * L, -1);
    if (dE == K_VERY_LARGE)
      weight *= 0;
    else
      weight *= exp(-c->beta * dE);
    for (int i = 1; i < L; i++) {
      const double Wi = gen_trials(c, r, chain + 3 * (i - 1), i, chain, chain + 3 * L, -1, tb1,
                                   tb2, w);
      weight *= Wi / T;
      if (weight <= 0 || r->overrun) break;
      const double rn = (double)rng_u32(r) / MT_MAX * Wi;
      int cb = 0;
      double cum = w[0];
      while (cum < rn && cb < T - 1) cum += w[++cb];
      for (int j = 0; j < 3; j++) chain[3 * i + j] = tb1[3 * cb + j];
      if (charged)
        for (int j = 0; j < 3; j++) chain[3 * (i + L) + j] = tb2[3 * cb + j];
    }
    total += weight * C;
  }
  free(chain);
  free(tb1);
  free(tb2);
  free(w);
  return total / (double)n_ins;
}

double po_chem_pot(po_ctx* c) {
  rng_t r = {&c->g, NULL, 0, 0, 0};
  return chem_pot_widom(c, &r, 50);
}

/* ForceField::CBMCFChainDeletion (cbmc.cc:330-442): the molecule to delete
 * or -1. */
static int chain_deletion(po_ctx* c, rng_t* r) {
  const int L = c->gc_chain_len, T = c->cbmc_trials;
  const int charged = c->gc_bead_charge != 0;
  int spc1, spc2;
  gc_species(c, &spc1, &spc2);
  int did = (int)floor((double)rng_u32(r) / MT_MAX * spc1);
  if (did >= spc1) did = spc1 - 1;
  if (r->overrun || did < 0) return -1;  /* nothing of the species to delete */
  did = c->phantom + c->coion + c->grafted + c->grafted_counterion + (charged ? did * (1 + L) : did);
  const int second = charged ? did + 1 : did;
  double* chain = (double*)calloc((size_t)6 * L, sizeof(double));
  double* tb1 = (double*)malloc(sizeof(double) * 3 * (size_t)T);
  double* tb2 = (double*)malloc(sizeof(double) * 3 * (size_t)T);
  double* w = (double*)malloc(sizeof(double) * (size_t)T);
  const double* x0 = c->x + 3 * c->mol_start[did];
  const double* s0 = c->x + 3 * c->mol_start[second];
  double weight = exp(-c->beta * po_beads_energy(c, x0, s0, 0, chain, chain + 3 * L, did));
  for (int j = 0; j < 3; j++) chain[j] = x0[j];
  if (charged)
    for (int j = 0; j < 3; j++) chain[3 * L + j] = s0[j];
  for (int i = 1; i < L && !r->overrun; i++) {
    for (int j = 0; j < 3; j++) chain[3 * i + j] = c->x[3 * (c->mol_start[did] + i) + j];
    if (charged)
      for (int j = 0; j < 3; j++)
        chain[3 * (i + L) + j] = c->x[3 * c->mol_start[did + i + 1] + j];
    gen_trials(c, r, chain + 3 * (i - 1), i, chain, chain + 3 * L, did, tb1, tb2, w);
    w[0] = exp(-c->beta * po_beads_energy(c, chain + 3 * i, chain + 3 * (charged ? i + L : i), i,
                                           chain, chain + 3 * L, did));
    double Wi = 0;
    for (int j = 0; j < T; j++) Wi += w[j];
    weight *= Wi / T;
  }
  free(chain);
  free(tb1);
  free(tb2);
  free(w);
  if (r->overrun) return -1;
  const int spc2_del = charged ? L : 0;
  double factorial = 1;
  for (int i = spc1; i > spc1 - 1; i--) factorial *= i;
  for (int i = spc2; i > spc2 - spc2_del; i--) factorial *= i;
  const double vol = c->box[0] * c->box[1] * c->box[2];
  double lam_over_vol = 1;
  lam_over_vol *= pow((c->debroglie / pow((double)L, 1.5)) / vol, 1);
  lam_over_vol *= pow((c->debroglie / pow(1.0, 1.5)) / vol, spc2_del);
  const double C = lam_over_vol * factorial;
  const double rn = (double)rng_u32(r) / MT_MAX;
  if (rn < C / (exp(c->beta * c->chem_pot) * weight)) return did;
  return -1;
}

/* Appends the grown chain (one molecule of L beads) and, for a charged
 * species, its L counterions (single-bead molecules), as the reference's
 * mols.push_back does (cbmc.cc:294-312). */
static void append_chain(po_ctx* c, const double* chain) {
  const int L = c->gc_chain_len, charged = c->gc_bead_charge != 0;
  const int add_b = charged ? 2 * L : L, add_m = charged ? 1 + L : 1;
  const int nb = c->n_bead + add_b, nm = c->n_mol + add_m;
  c->x = (double*)realloc(c->x, sizeof(double) * 3 * (size_t)nb);
  c->t = (double*)realloc(c->t, sizeof(double) * 3 * (size_t)nb);
  c->q = (double*)realloc(c->q, sizeof(double) * (size_t)nb);
  c->type = (int*)realloc(c->type, sizeof(int) * (size_t)nb);
  c->mol_start = (int*)realloc(c->mol_start, sizeof(int) * (size_t)(nm + 1));
  c->bond_mol = (double*)realloc(c->bond_mol, sizeof(double) * (size_t)nm);
  for (int i = 0; i < add_b; i++) {
    const int b = c->n_bead + i;
    for (int j = 0; j < 3; j++) c->x[3 * b + j] = c->t[3 * b + j] = chain[3 * i + j];
    c->q[b] = i < L ? c->gc_bead_charge : -c->gc_bead_charge;
    c->type[b] = c->gc_type;
  }
  int m = c->n_mol;
  c->mol_start[m + 1] = c->n_bead + L;
  for (int i = 1; i < add_m; i++) c->mol_start[m + 1 + i] = c->n_bead + L + i;
  for (int i = 0; i < add_m; i++) c->bond_mol[m + i] = 0;
  c->n_bead = nb;
  c->n_mol = nm;
}

/* Erases molecules [m0, m0 + count) (simulation.cc:383-391). */
static void erase_mols(po_ctx* c, int m0, int count) {
  const int b0 = c->mol_start[m0], b1 = c->mol_start[m0 + count], nb = b1 - b0;
  memmove(c->x + 3 * b0, c->x + 3 * b1, sizeof(double) * 3 * (size_t)(c->n_bead - b1));
  memmove(c->t + 3 * b0, c->t + 3 * b1, sizeof(double) * 3 * (size_t)(c->n_bead - b1));
  memmove(c->q + b0, c->q + b1, sizeof(double) * (size_t)(c->n_bead - b1));
  memmove(c->type + b0, c->type + b1, sizeof(int) * (size_t)(c->n_bead - b1));
  for (int m = m0; m + count <= c->n_mol; m++) c->mol_start[m] = c->mol_start[m + count] - nb;
  memmove(c->bond_mol + m0, c->bond_mol + m0 + count,
          sizeof(double) * (size_t)(c->n_mol - m0 - count));
  c->n_bead -= nb;
  c->n_mol -= count;
}

/* Simulation::GCMove (simulation.cc:357-404); move type 5 insertion, 6
 * deletion. After an accepted exchange the running totals are recomputed
 * (the reference updates them incrementally; the totals agree to
 * round-off). */
static int gc_move(po_ctx* c, rng_t* r, int* acc) {
  *acc = 0;
  const int insert = (int)(rng_u32(r) % 2u);
  if (insert) {
    double* chain = (double*)calloc((size_t)6 * c->gc_chain_len, sizeof(double));
    const int ok = chain_insertion(c, r, chain);
    if (ok && !r->overrun) {
      append_chain(c, chain);
      *acc = 1;
    }
    free(chain);
  } else if (c->n_mol - c->phantom - c->coion > 0) {
    const int did = chain_deletion(c, r);
    if (did >= c->phantom + c->coion) {
      int ions = 0;
      for (int b = c->mol_start[did]; b < c->mol_start[did + 1]; b++)
        ions += (int)round(fabs(c->q[b]));
      erase_mols(c, did, 1 + ions);
      *acc = 1;
    }
  }
  if (*acc) {
    update_counts(c);
    po_total_energy(c, NULL);
  }
  return insert ? 5 : 6;
}

void po_coords(const po_ctx* c, double* out) {
  memcpy(out, c->x, sizeof(double) * 3 * (size_t)c->n_bead);
}

void po_set_coords(po_ctx* c, const double* xyz) {
  memcpy(c->x, xyz, sizeof(double) * 3 * (size_t)c->n_bead);
  memcpy(c->t, xyz, sizeof(double) * 3 * (size_t)c->n_bead);
  po_total_energy(c, NULL);
}

/* RadiusOfGyration / RadiusOfGyrationXYZ / EndToEndDistance
 * (simulation.cc:406-500). */
/* ------------------------------------------------ wall-force pressure */
/* PotentialTruncatedLJ::PairForce (potential_truncated_lj.cc:87-122): beyond
 * a positive cut-off it returns the cut-off's r^-6 term at r, as the
 * reference does; hard spheres have no force (potential_hard_sphere.cc:51-56). */
static double lj_force(const po_ctx* c, const double* a, int ta, const double* b, int tb) {
  if (c->pair_kind == 1) return 0;
  double r = bbdist(a, b, c->box, c->npbc);
  double sigma = (c->lj_sig[ta] + c->lj_sig[tb]) / 2;
  double epsilon = sqrt((c->lj_eps[ta] * c->lj_eps[tb]));
  double r6;
  if (r <= 0) return K_VERY_LARGE;
  if (c->lj_cut < 0) {
    if (r < K216 * sigma) {
      r6 = pow((sigma / r), 6);
      return 4 * epsilon * (r6 * r6 * 12 / r - r6 * 6 / r);
    }
    return 0;
  }
  if (r < c->lj_cut)
    r6 = pow((sigma / r), 6);
  else
    r6 = pow((sigma / c->lj_cut), 6);
  return 4 * epsilon * (r6 * r6 * 12 / r - r6 * 6 / r);
}

/* GetDistVector (misc.cc:43-56): from b1 to b2, wrapped on periodic axes. */
static void dist_vec(const double* b1, const double* b2, const double* box, int npbc,
                     double* r) {
  for (int i = 0; i < 3; i++) {
    double di = b2[i] - b1[i];
    if (i < npbc) di -= box[i] * round(di / box[i]);
    r[i] = di;
  }
}

/* PotentialEwaldCoul::PairForceZReal (potential_ewald_coul.cc:261-293): the
 * z force on wall charge a from bead b, real space over the image cells. */
static double ew_force_z_real(const po_ctx* c, const double* a, double qa, const double* b,
                              double qb) {
  double force_z = 0;
  if (qa * qb == 0) return force_z;
  double r[3];
  dist_vec(b, a, c->ebox, c->npbc, r);
  double prefactor = c->lB * qa * qb;
  double prefactor2 = 2 * sqrt(c->alpha / K_PI);
  for (int i = -c->real_cell[0]; i <= c->real_cell[0]; i++)
    for (int j = -c->real_cell[1]; j <= c->real_cell[1]; j++)
      for (int k = -c->real_cell[2]; k <= c->real_cell[2]; k++) {
        double v[3] = {r[0] + i * c->ebox[0], r[1] + j * c->ebox[1], r[2] + k * c->ebox[2]};
        double d = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (d > 0 && d <= c->real_cut)
          force_z += prefactor * ((prefactor2 * exp(-c->alpha * d * d)) +
                                  (erfc(sqrt(c->alpha) * d) / d)) * v[2] / (d * d);
      }
  return force_z;
}

/* PotentialEwaldCoul::PairForceZRepl (potential_ewald_coul.cc:297-324): the
 * reference sums k_z e^{-k^2/4a}/k^2 sin(k.r) over the whole k cube; the
 * summand is even under k -> -k, so here twice the half space. */
static double ew_force_z_repl(const po_ctx* c, const double* a, double qa, const double* b,
                              double qb) {
  if (qa * qb == 0) return 0;
  double r[3];
  dist_vec(b, a, c->ebox, c->npbc, r);
  double prefactor = c->lB * 4 * K_PI * qa * qb / c->evol;
  double f = 0;
  for (int k = 0; k < c->n_k; k++) {
    const double* kv = c->kv + 3 * k;
    f += kv[2] * c->kw[k] * sin(kv[0] * r[0] + kv[1] * r[1] + kv[2] * r[2]);
  }
  return prefactor * 2 * f;
}

/* PotentialTruncatedLJWall::BeadForceOnWall (potential_truncated_lj_wall.cc:
 * 136-214); the hard and square-well walls have none. */
static double wall_force(const po_ctx* c, double z, int ty) {
  if (c->ext_kind != 0) return 0;
  double force = 0;
  double sigma = c->wall_sig[ty], epsilon = c->wall_eps[ty];
  double R0 = 3 * K213 * sigma, K = 1, lz = c->box[2], mc = c->wall_cut;
  const double k93 = 2.59807621135;
  int g = c->graft[ty];
  if (epsilon == 0) return 0;
  if (z <= 0 || z >= lz) return K_VERY_LARGE;
  if (mc < 0 && g == 0) {
    if (z < K213 * sigma) {
      double r3 = pow((sigma / z), 3);
      force += k93 * epsilon * (r3 * r3 * 6 / z - r3 * 3 / z);
    }
    if (lz - z < K213 * sigma) {
      double r3 = pow((sigma / (lz - z)), 3);
      force += k93 * epsilon * (r3 * r3 * 6 / (lz - z) - r3 * 3 / (lz - z));
    }
  } else if (g == 1) {
    double r3 = pow((sigma / z), 3);
    force += k93 * epsilon * (r3 * r3 * 6 / z - r3 * 3 / z);
    force += -K * R0 * z / (1 - pow(z / R0, 2));
    if (lz - z < K213 * sigma) {
      r3 = pow((sigma / (lz - z)), 3);
      force += k93 * epsilon * (r3 * r3 * 6 / (lz - z) - r3 * 3 / (lz - z));
    }
  } else if (g == 2) {
    double r3 = pow((sigma / (lz - z)), 3);
    force += k93 * epsilon * (r3 * r3 * 6 / (lz - z) - r3 * 3 / (lz - z));
    force += -K * R0 * (lz - z) / (1 - pow((lz - z) / R0, 2));
    if (z < K213 * sigma) {
      r3 = pow((sigma / z), 3);
      force += k93 * epsilon * (r3 * r3 * 6 / z - r3 * 3 / z);
    }
  } else {
    double r3 = pow((sigma / (z < mc ? z : mc)), 3);
    force += k93 * epsilon * (r3 * r3 * 6 / z - r3 * 3 / z);
    if (lz - z < mc) {
      r3 = pow((sigma / (lz - z)), 3);
      force += k93 * epsilon * (r3 * r3 * 6 / (lz - z) - r3 * 3 / (lz - z));
    } else {
      r3 = pow((sigma / mc), 3);
      force += k93 * epsilon * (r3 * r3 * 6 / z - r3 * 3 / z);
    }
  }
  return force;
}

/* The pieces, for the checks against the reference: the wall force of bead
 * i, and the real / reciprocal z force on bead a from bead b. */
double po_wall_force(const po_ctx* c, int i) { return wall_force(c, c->x[3 * i + 2], c->type[i]); }

void po_ewald_force_z(const po_ctx* c, int a, int b, double* out2) {
  out2[0] = ew_force_z_real(c, c->x + 3 * a, c->q[a], c->x + 3 * b, c->q[b]);
  out2[1] = ew_force_z_repl(c, c->x + 3 * a, c->q[a], c->x + 3 * b, c->q[b]);
}

/* The oracle's configuration and parameters of the wall-force pressure, for
 * harnesses that run another implementation of it on the same inputs. */
void po_slit_inputs(const po_ctx* c, double* scal, double* per_type, int* type, double* q,
                    int* mol_start, double* kv, double* kw) {
  if (scal) {
    double v[26] = {c->box[0], c->box[1], c->box[2], c->ebox[0], c->ebox[1], c->ebox[2],
                    c->npbc, c->phantom, c->use_pair, c->use_ewald, c->use_ext,
                    c->pair_kind, c->ext_kind, c->lj_cut, c->lB, c->alpha, c->real_cut,
                    c->real_cell[0], c->real_cell[1], c->real_cell[2], c->evol,
                    c->wall_cut, c->n_type, c->n_k, c->n_bead, c->n_mol};
    memcpy(scal, v, sizeof v);
  }
  if (per_type)
    for (int t = 0; t < c->n_type; t++) {
      per_type[5 * t] = c->lj_sig[t];
      per_type[5 * t + 1] = c->lj_eps[t];
      per_type[5 * t + 2] = c->wall_sig[t];
      per_type[5 * t + 3] = c->wall_eps[t];
      per_type[5 * t + 4] = c->graft[t];
    }
  if (type) memcpy(type, c->type, sizeof(int) * (size_t)c->n_bead);
  if (q) memcpy(q, c->q, sizeof(double) * (size_t)c->n_bead);
  if (mol_start) memcpy(mol_start, c->mol_start, sizeof(int) * (size_t)(c->n_mol + 1));
  if (kv) memcpy(kv, c->kv, sizeof(double) * 3 * (size_t)c->n_k);
  if (kw) memcpy(kw, c->kw, sizeof(double) * (size_t)c->n_k);
}

/* ForceField::CalcPressureForceLJELSlit (pressure.cc:400-488) on the current
 * configuration: wall sites (the first phantom molecules, half on each wall)
 * against the system, plus the 9-3 wall forces; out12 = p_tensor[0..11]
 * (0-5 the averages the stat file prints, 6-11 the accumulators). */
void po_pressure_force_slit(po_ctx* c, double* out12) {
  double* p = c->p_tensor;
  c->vp_z += 1;
  const int ph = c->phantom, nm = c->n_mol;
  for (int i = 0; i < ph; i++) {
    const int wi = c->mol_start[i];
    for (int j = ph / 2; j < nm; j++)
      for (int k = c->mol_start[j]; k < c->mol_start[j + 1]; k++) {
        double C;
        if (i < ph / 2 && j >= ph)
          C = -0.5;
        else if (i < ph && j >= ph)
          C = 0.5;
        else
          C = -1;
        int k_id = 2;
        if (j >= ph) k_id = (c->mol_start[j + 1] - c->mol_start[j] > 1) ? 1 : 0;
        if (c->use_pair && (i < ph / 2 || j >= ph)) {
          double r[3];
          dist_vec(c->x + 3 * k, c->x + 3 * wi, c->box, c->npbc, r);
          double zc = r[2] / sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
          double f = C * zc * lj_force(c, c->x + 3 * k, c->type[k], c->x + 3 * wi, c->type[wi]);
          if (k_id == 0)
            p[6] += f;
          else if (k_id == 1)
            p[7] += f;
          else if (k_id == 2 && c->vp_z == 1)
            p[8] += f;
        }
        if (c->use_ewald && (i < ph / 2 || j >= ph)) {
          double f = C * ew_force_z_real(c, c->x + 3 * wi, c->q[wi], c->x + 3 * k, c->q[k]);
          f += C * ew_force_z_repl(c, c->x + 3 * wi, c->q[wi], c->x + 3 * k, c->q[k]);
          if (k_id == 0)
            p[9] += f;
          else if (k_id == 1)
            p[10] += f;
          else if (k_id == 2 && c->vp_z == 1)
            p[11] += f;
        }
      }
  }
  if (c->use_ext)
    for (int i = ph; i < nm; i++)
      for (int j = c->mol_start[i]; j < c->mol_start[i + 1]; j++) {
        double f = 0.5 * wall_force(c, c->x[3 * j + 2], c->type[j]);
        if (c->mol_start[i + 1] - c->mol_start[i] > 1)
          p[7] += f;
        else
          p[6] += f;
      }
  const double area = c->box[0] * c->box[1];
  if (c->vp_z == 1) {
    p[2] = p[8] / area;
    p[5] = p[11] / area;
  }
  p[0] = p[6] / (c->vp_z * area);
  p[1] = p[7] / (c->vp_z * area);
  p[3] = p[9] / (c->vp_z * area);
  p[4] = p[10] / (c->vp_z * area);
  if (out12) memcpy(out12, p, 12 * sizeof(double));
}

void po_observables(const po_ctx* c, double* out) {
  double rg = 0, rx = 0, ry = 0, rz = 0, ete = 0;
  for (int m = 0; m < c->n_mol; m++) {
    int b0 = c->mol_start[m], n = c->mol_start[m + 1] - b0;
    if (n <= 1) continue;
    double g = 0, gx = 0, gy = 0, gz = 0;
    for (int j = 0; j < n - 1; j++)
      for (int k = j + 1; k < n; k++) {
        double r = bbdist(c->x + 3 * (b0 + j), c->x + 3 * (b0 + k), c->box, 0);
        g += r * r;
        double x = fabs(CX(b0 + j, 0) - CX(b0 + k, 0));
        double y = fabs(CX(b0 + j, 1) - CX(b0 + k, 1));
        double z = fabs(CX(b0 + j, 2) - CX(b0 + k, 2));
        gx += x * x, gy += y * y, gz += z * z;
      }
    rg += g / (n * n), rx += gx / (n * n), ry += gy / (n * n), rz += gz / (n * n);
    double e = bbdist(c->x + 3 * b0, c->x + 3 * (b0 + n - 1), c->box, 0);
    ete += e * e;
  }
  int nc = c->grafted + c->n_chain;
  if (nc > 0) rg /= nc, rx /= nc, ry /= nc, rz /= nc, ete /= nc;
  out[0] = rg, out[1] = rx, out[2] = ry, out[3] = rz, out[4] = ete;
}

/* CalcRhoZ (simulation.cc:1029-1045), one pass on a zeroed histogram. */
int po_rhoz(const po_ctx* c, double* out, int cap) {
  double res = 0.02;
  int nb = (int)ceil(c->box[2] / res);
  int n = 3 * nb < cap ? 3 * nb : cap;
  for (int i = 0; i < n; i++) out[i] = 0;
  for (int m = c->phantom; m < c->n_mol; m++) {
    int b0 = c->mol_start[m], sz = c->mol_start[m + 1] - b0;
    int id = sz > 1 ? 0 : (c->q[b0] >= 0 ? 1 : 2);
    for (int j = b0; j < b0 + sz; j++) {
      double z = c->x[3 * j + 2];
      z -= c->box[2] * floor(z / c->box[2]);
      int bz = (int)floor(z / res);
      if (bz >= 0 && bz < nb && 3 * bz + id < n)
        out[3 * bz + id] += 1.0 / (c->box[0] * c->box[1] * res);
    }
  }
  return nb;
}

/* ForceField::BeadsEnergy (cbmc.cc:5-151): energy of a trial chain bead b1
 * (and, for a charged species, its trial counterion b2) against the system
 * minus the molecules being deleted, the first current_len grown beads (and
 * their counterions), each other, the walls, and in Ewald the self terms and
 * the dipole change. LJ with the immediately preceding grown bead is left out
 * (cbmc.cc:57-58). The reciprocal part is written with S(k) of the "other"
 * charges: sum over the pairs + half the self pairs = (4 pi lB / V) sum_half
 * e^{-k^2/4a}/k^2 (|S_o + q1 e1 + q2 e2|^2 - |S_o|^2). */
double po_beads_energy(po_ctx* c, const double* b1, const double* b2, int cl,
                       const double* chain, const double* chain_ci, int delete_id) {
  const int charged = c->gc_bead_charge != 0;
  const double q1 = c->gc_bead_charge, q2 = -c->gc_bead_charge;
  const int t = c->gc_type;
  const int L = c->gc_chain_len;
  int d_lo = -1, d_hi = -1; /* excluded molecules [d_lo, d_hi] */
  if (delete_id >= 0) {
    d_lo = delete_id;
    d_hi = delete_id + (charged ? L : 0);
  }
  double pair_e = 0, ew = 0;
  for (int m = 0; m < c->n_mol; m++) {
    if (m >= d_lo && m <= d_hi) continue;
    for (int j = c->mol_start[m]; j < c->mol_start[m + 1]; j++) {
      const double* pj = c->x + 3 * j;
      if (c->use_pair) {
        pair_e += lj_pair(c, b1, t, pj, c->type[j]);
        if (charged) pair_e += lj_pair(c, b2, t, pj, c->type[j]);
      }
      if (c->use_ewald) {
        ew += ew_real_pair(c, b1, q1, pj, c->q[j]);
        if (charged) ew += ew_real_pair(c, b2, q2, pj, c->q[j]);
      }
    }
  }
  for (int i = 0; i < cl; i++) {
    const double* ci = chain + 3 * i;
    const double* cc = charged ? chain_ci + 3 * i : NULL;
    if (c->use_pair) {
      if (i < cl - 1) pair_e += lj_pair(c, b1, t, ci, t);
      if (charged) {
        pair_e += lj_pair(c, b1, t, cc, t);
        pair_e += lj_pair(c, b2, t, ci, t);
        pair_e += lj_pair(c, b2, t, cc, t);
      }
    }
    if (c->use_ewald) {
      ew += ew_real_pair(c, b1, q1, ci, q1);
      if (charged) {
        ew += ew_real_pair(c, b1, q1, cc, q2);
        ew += ew_real_pair(c, b2, q2, ci, q1);
        ew += ew_real_pair(c, b2, q2, cc, q2);
      }
    }
  }
  if (c->use_pair && charged) pair_e += lj_pair(c, b1, t, b2, t);
  if (c->use_ewald && pair_e < K_VERY_LARGE) {
    ew += ew_self(c, q1) + 0.5 * ew_real_pair(c, b1, q1, b1, q1);
    if (charged) {
      ew += ew_self(c, q2) + ew_real_pair(c, b1, q1, b2, q2) + 0.5 * ew_real_pair(c, b2, q2, b2, q2);
    }
    double* so = (double*)calloc((size_t)2 * (c->n_k > 0 ? c->n_k : 1), sizeof(double));
    double* sn = (double*)calloc((size_t)2 * (c->n_k > 0 ? c->n_k : 1), sizeof(double));
    double mz = 0;
    for (int m = 0; m < c->n_mol; m++) {
      if (m >= d_lo && m <= d_hi) continue;
      for (int j = c->mol_start[m]; j < c->mol_start[m + 1]; j++) {
        sk_add(c, c->x + 3 * j, c->q[j], 1.0, so);
        mz += c->q[j] * c->x[3 * j + 2];
      }
    }
    for (int i = 0; i < cl; i++) {
      sk_add(c, chain + 3 * i, q1, 1.0, so);
      mz += q1 * chain[3 * i + 2];
      if (charged) {
        sk_add(c, chain_ci + 3 * i, q2, 1.0, so);
        mz += q2 * chain_ci[3 * i + 2];
      }
    }
    memcpy(sn, so, sizeof(double) * 2 * (size_t)c->n_k);
    sk_add(c, b1, q1, 1.0, sn);
    if (charged) sk_add(c, b2, q2, 1.0, sn);
    ew += sk_energy(c, sn) - sk_energy(c, so);
    if (c->dipole) {
      double mzn = mz + q1 * b1[2] + (charged ? q2 * b2[2] : 0.0);
      ew += c->lB * 2 * K_PI / (c->evol / 1.0) * (mzn * mzn - mz * mz);
    }
    free(so);
    free(sn);
  }
  if (c->use_ext) {
    pair_e += wall_energy(c, b1[2], t);
    if (charged) pair_e += wall_energy(c, b2[2], t);
  }
  if (pair_e >= K_VERY_LARGE) return K_VERY_LARGE;
  return pair_e + ew;
}
