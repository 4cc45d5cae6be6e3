/* CPU oracle: plain-C restatement of the reference's MPCD + microswimmer step.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and bench.py's CPU
 * baseline as the checker.  It restates, in the same operation order, the
 * reference code cited at each function (paths relative to the reference
 * project).  Its parity is pinned by tests against fixtures that
 * oracle/_ref/ref_harness produced from the reference's own sources.
 */
#define _POSIX_C_SOURCE 200809L
#include "mpcd_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846 /* src/libcilia/abbrev.cpp:9 */

/* ------------------------------------------------------------ MT19937 -- */
/* Matsumoto & Nishimura (1998) generator, as used through MTRand
 * (src/libcilia/MersenneTwister.h:146-162 seeding, :197-226 output). */
typedef struct {
  uint32_t mt[624];
  int idx;
} mt_t;

static void mt_seed(mt_t* g, uint32_t s) {
  g->mt[0] = s;
  for (int i = 1; i < 624; ++i)
    g->mt[i] = (uint32_t)(1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i);
  g->idx = 624;
}

static void mt_twist(mt_t* g) {
  for (int i = 0; i < 624; ++i) {
    uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
    uint32_t v = g->mt[(i + 397) % 624] ^ (y >> 1);
    if (y & 1u) v ^= 0x9908b0dfu;
    g->mt[i] = v;
  }
  g->idx = 0;
}

static uint32_t mt_u32(mt_t* g) {
  if (g->idx >= 624) mt_twist(g);
  uint32_t y = g->mt[g->idx++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

/* MTRand::rand() in [0,1] (MersenneTwister.h:153-154) */
static double mt_rand(mt_t* g) { return (double)mt_u32(g) * (1.0 / 4294967295.0); }
/* MTRand::randDblExc() in (0,1) (MersenneTwister.h:165-166); rnd() (basicf.h:27-34) */
static double mt_dblexc(mt_t* g) { return ((double)mt_u32(g) + 0.5) * (1.0 / 4294967296.0); }
/* normalrand(): Box-Muller, cosine branch (src/libcilia/basicf.h:52-62) */
static double mt_normal(mt_t* g) {
  double x1 = mt_dblexc(g);
  double x2 = mt_dblexc(g);
  return sqrt(-2.0 * log(x1)) * cos(2.0 * ORC_PI * x2);
}
/* rgamma(Nc): Marsaglia-Tsang Gamma(3(Nc-1)/2, 1) (src/libcilia/mpcd.cpp:13-43) */
static double mt_gamma(mt_t* g, int nc) {
  const double d = 1.5 * nc - 1.833333333333333333333333333333333;
  const double c = 0.33333333333333333333333333333333 / sqrt(d);
  double x, v;
  for (;;) {
    do {
      x = mt_normal(g);
      v = 1.0 + c * x;
    } while (v <= 0.0);
    v = v * v * v;
    double u = mt_dblexc(g), x2 = x * x, x4 = x2 * x2;
    if (u < 1.0 - 0.0331 * x4) return d * v;
    if (log(u) < 0.5 * x2 + d * (1.0 - v + log(v))) return d * v;
  }
}

/* ------------------------------------------------------------- objects -- */
enum { OBJ_SPHERE = 0, OBJ_CILIA = 1, OBJ_CBCILIA = 2, OBJ_CLAMI = 3 };

typedef struct {
  int cil_obj, sphere_bead, rod, bead;
  double l0;
} attach_t;

typedef struct {
  int kind;
  int rods, len, startidx;
  long boff; /* offset of bead (rod 0, bead 0) in the global bead arrays */
  double k;
  /* sphere (src/sphere.h:46-57) */
  double radius, headbond;
  int npart;
  int (*neilist)[7];
  /* cilia (src/cilia.h:54-81) */
  double beatstrength, bending, min_bend, max_bend, m_speed, midpnt, start, tstroke;
  int num_anker;
  double *newlength, *oldlength;
  double power_dur, recovery_dur;
  /* clami (src/clami.h:108-114) */
  int sphere_obj, ncil;
  int* cil_objs;
  attach_t* springs;
  int nspr;
} obj_t;

struct orc_sim {
  int L[3];
  long ncell;
  double tstep, ststep, globalt;
  double a[3];
  long double diss;
  mt_t rng;
  int threads;
  mt_t* trng; /* per-thread generators (threads > 1) */
  /* fluid (src/libcilia/fluid.h:33-34): mass 1 */
  long n;
  double *pos, *vel;
  /* beads of all objects, md_objects order, rod-major */
  long nb;
  double *bpos, *bvel, *bfrc, *bmass;
  int nobj;
  obj_t* objs;
  /* cell lists: fluid in index order, then beads (src/libcilia/mpcd.cpp:257-267) */
  int* cell_of;
  long* cstart;
  long* members;
  double* l_energy;
  /* boundaries and body force (-DNOSLIP / -DSLIP, -DFLUID_FLOW_G in the reference) */
  int walls;            /* 0 periodic, 1 no-slip, 2 slip walls at z = 0 and z = Lz - 1 */
  double gravity, omega;
  /* contact forces between cilia (-DREPELLING=eps in the reference); 0 = off */
  double repelling;
  long contacts; /* section pairs found within the cutoff since orc_set_repelling */
};

/* ---------------------------------------------------------------- setup -- */
orc_sim* orc_create(int lx, int ly, int lz, double tstep, double ststep, unsigned int seed) {
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  s->L[0] = lx;
  s->L[1] = ly;
  s->L[2] = lz;
  s->ncell = (long)lx * ly * lz;
  s->tstep = tstep;
  s->ststep = ststep;
  s->threads = 1;
  mt_seed(&s->rng, seed);
  s->cstart = (long*)calloc(s->ncell + 1, sizeof(long));
  s->l_energy = (double*)calloc(s->ncell, sizeof(double));
  return s;
}

static void obj_free(obj_t* o) {
  free(o->neilist);
  free(o->newlength);
  free(o->oldlength);
  free(o->cil_objs);
  free(o->springs);
}

void orc_destroy(orc_sim* s) {
  if (!s) return;
  for (int i = 0; i < s->nobj; ++i) obj_free(&s->objs[i]);
  free(s->objs);
  free(s->pos);
  free(s->vel);
  free(s->bpos);
  free(s->bvel);
  free(s->bfrc);
  free(s->bmass);
  free(s->cell_of);
  free(s->cstart);
  free(s->members);
  free(s->l_energy);
  free(s->trng);
  free(s);
}

unsigned int orc_mt_next(orc_sim* s) { return mt_u32(&s->rng); }
double orc_rgamma(orc_sim* s, int nc) { return mt_gamma(&s->rng, nc); }

void orc_init_shift(orc_sim* s) {
  for (int q = 0; q < 3; ++q) s->a[q] = mt_dblexc(&s->rng); /* mpcd.cpp:92-95 */
}
void orc_set_shift(orc_sim* s, const double* a3) { memcpy(s->a, a3, sizeof s->a); }
void orc_get_shift(const orc_sim* s, double* a3) { memcpy(a3, s->a, sizeof s->a); }
void orc_set_globalt(orc_sim* s, double t) { s->globalt = t; }
double orc_get_globalt(const orc_sim* s) { return s->globalt; }

static void alloc_fluid(orc_sim* s, long n) {
  free(s->pos);
  free(s->vel);
  s->n = n;
  s->pos = (double*)calloc(3 * (size_t)n, sizeof(double));
  s->vel = (double*)calloc(3 * (size_t)n, sizeof(double));
}

/* Fluid::create (src/libcilia/fluid.cpp:55-98): positions rnd()*L, velocities
 * normalrand()*sqrt(kT) with kT = 1, centre-of-mass velocity removed. */
void orc_fluid_create(orc_sim* s) {
  long n = s->ncell * 10; /* rho = 10 (mpcd.h:69; fluid.cpp:24) */
  alloc_fluid(s, n);
  for (long i = 0; i < n; ++i) {
    for (int q = 0; q < 3; ++q) s->pos[3 * i + q] = mt_dblexc(&s->rng) * (double)s->L[q] * 1.0;
    for (int q = 0; q < 3; ++q) s->vel[3 * i + q] = mt_normal(&s->rng) * sqrt(1.0);
  }
  double cm[3] = {0.0, 0.0, 0.0};
  for (long i = 0; i < n; ++i)
    for (int q = 0; q < 3; ++q) cm[q] += s->vel[3 * i + q];
  for (int q = 0; q < 3; ++q) cm[q] /= n;
  for (long i = 0; i < n; ++i)
    for (int q = 0; q < 3; ++q) s->vel[3 * i + q] -= cm[q];
}

int orc_fluid_set(orc_sim* s, long n, const double* pos, const double* vel) {
  alloc_fluid(s, n);
  memcpy(s->pos, pos, 3 * (size_t)n * sizeof(double));
  memcpy(s->vel, vel, 3 * (size_t)n * sizeof(double));
  return 0;
}
long orc_fluid_count(const orc_sim* s) { return s->n; }
void orc_fluid_get(const orc_sim* s, double* pos, double* vel) {
  if (pos) memcpy(pos, s->pos, 3 * (size_t)s->n * sizeof(double));
  if (vel) memcpy(vel, s->vel, 3 * (size_t)s->n * sizeof(double));
}

static obj_t* new_obj(orc_sim* s, int kind, int rods, int len) {
  s->objs = (obj_t*)realloc(s->objs, (size_t)(s->nobj + 1) * sizeof(obj_t));
  obj_t* o = &s->objs[s->nobj++];
  memset(o, 0, sizeof *o);
  o->kind = kind;
  o->rods = rods;
  o->len = len;
  o->boff = s->nb;
  long add = (long)rods * len;
  if (add > 0) {
    long nb = s->nb + add;
    s->bpos = (double*)realloc(s->bpos, 3 * (size_t)nb * sizeof(double));
    s->bvel = (double*)realloc(s->bvel, 3 * (size_t)nb * sizeof(double));
    s->bfrc = (double*)realloc(s->bfrc, 3 * (size_t)nb * sizeof(double));
    s->bmass = (double*)realloc(s->bmass, (size_t)nb * sizeof(double));
    memset(s->bpos + 3 * s->nb, 0, 3 * (size_t)add * sizeof(double));
    memset(s->bvel + 3 * s->nb, 0, 3 * (size_t)add * sizeof(double));
    memset(s->bfrc + 3 * s->nb, 0, 3 * (size_t)add * sizeof(double));
    memset(s->bmass + s->nb, 0, (size_t)add * sizeof(double));
    s->nb = nb;
  }
  return o;
}

static inline double* BP(orc_sim* s, const obj_t* o, int r, int j) { return s->bpos + 3 * (o->boff + (long)r * o->len + j); }
static inline double* BV(orc_sim* s, const obj_t* o, int r, int j) { return s->bvel + 3 * (o->boff + (long)r * o->len + j); }
static inline double* BF(orc_sim* s, const obj_t* o, int r, int j) { return s->bfrc + 3 * (o->boff + (long)r * o->len + j); }

static double sqdist3(const double* a, const double* b) {
  double d = 0.0;
  for (int i = 0; i < 3; ++i) {
    double t = a[i] - b[i];
    d += t * t;
  }
  return d;
}

/* Sphere::create_neillist (src/sphere.cpp:264-285) */
static void sphere_neilist(orc_sim* s, obj_t* o, int max_part) {
  const double rcutsq = 1.1 * 1.1;
  for (int j = 0; j < max_part + 1; ++j)
    for (int k = 0; k < 7; ++k) o->neilist[j][k] = 0;
  for (int j = 1; j < max_part; ++j)
    for (int k = j + 1; k < max_part + 1; ++k)
      if (sqdist3(BP(s, o, 0, j), BP(s, o, 0, k)) < rcutsq) {
        o->neilist[j][0] += 1;
        o->neilist[k][0] += 1;
        o->neilist[j][o->neilist[j][0]] = k;
        o->neilist[k][o->neilist[k][0]] = j;
      }
}

/* Sphere::create (src/sphere.cpp:136-262): icosahedron refined fill_factor
 * times by edge midpoints, rotated 90 degrees about y, projected on `radius`. */
static void sphere_create(orc_sim* s, obj_t* o, double wx, double wy, double wz, int fill) {
  const double c5 = cos(2.0 * ORC_PI / 5), s5 = sin(2.0 * ORC_PI / 5);
  const double c45 = cos(ORC_PI - 2.0 * 2.0 * ORC_PI / 5), s45 = sin(ORC_PI - 2.0 * 2.0 * ORC_PI / 5);
  const double ico[13][3] = {{0, 0, 0},
                             {0., 0., 1.13},
                             {c5, s5, 0.50230},
                             {-c45, s45, 0.50230},
                             {-c45, -s45, 0.5023},
                             {c5, -s5, 0.50230},
                             {1.0, 0.0, 0.5023},
                             {c45, s45, -0.5023},
                             {-c5, s5, -0.5023},
                             {-1.0, 0.0, -0.5023},
                             {-c5, -s5, -0.5023},
                             {cos(ORC_PI - 4.0 * ORC_PI / 5), -s45, -0.5023},
                             {0., 0., -1.13}};
  for (int i = 1; i < 13; ++i)
    for (int q = 0; q < 3; ++q) BP(s, o, 0, i)[q] = ico[i][q] * 0.8513;
  int npart = 12, tel = 12;
  for (int it = 0; it < fill; ++it) {
    sphere_neilist(s, o, npart);
    for (int j = 1; j < npart; ++j)
      for (int k = j + 1; k < npart + 1; ++k)
        for (int l = 1; l < o->neilist[j][0] + 1; ++l)
          if (o->neilist[j][l] == k) {
            tel += 1;
            for (int q = 0; q < 3; ++q) BP(s, o, 0, tel)[q] = (BP(s, o, 0, j)[q] + BP(s, o, 0, k)[q]) / 2.0;
          }
    npart = tel;
    for (int i = 1; i < npart + 1; ++i)
      for (int q = 0; q < 3; ++q) BP(s, o, 0, i)[q] *= 2.0;
  }
  sphere_neilist(s, o, npart);
  npart++;
  for (int i = 1; i < npart; ++i) {
    double* p = BP(s, o, 0, i);
    double xi = p[0], zi = p[2];
    p[0] = zi;
    p[2] = -xi;
  }
  for (int i = 1; i < npart; ++i) {
    double* p = BP(s, o, 0, i);
    double scale = o->radius / sqrt(sqdist3(p, BP(s, o, 0, 0)));
    for (int q = 0; q < 3; ++q) p[q] *= scale;
    p[0] = p[0] + wx;
    p[1] += wy;
    p[2] = p[2] + wz;
  }
  BP(s, o, 0, 0)[0] += wx;
  BP(s, o, 0, 0)[1] += wy;
  BP(s, o, 0, 0)[2] += wz;
  double hb = 0.0, norm = 0.0;
  for (int i = 1; i < npart; ++i)
    for (int j = 1; j < o->neilist[i][0] + 1; ++j) {
      hb += sqrt(sqdist3(BP(s, o, 0, i), BP(s, o, 0, o->neilist[i][j])));
      norm++;
    }
  o->headbond = hb / norm;
}

int orc_add_sphere(orc_sim* s, double radius, double k, double x, double y, double z, int npart) {
  int fill = npart == 163 ? 2 : (npart == 643 ? 3 : 0); /* sphere.cpp:17-26 */
  if (fill == 0) return -1;
  obj_t* o = new_obj(s, OBJ_SPHERE, 1, npart);
  o->radius = radius;
  o->k = k;
  o->npart = npart;
  o->startidx = 0;
  o->neilist = (int(*)[7])calloc((size_t)npart, sizeof(int[7]));
  sphere_create(s, o, x, y, z, fill);
  return s->nobj - 1;
}

/* Cilia::create (src/cilia.cpp:275-325): three filaments at bond length 0.5,
 * rotated by (thetaX, thetaY, thetaZ) and translated to (wx, wy, wz). */
static void cilia_create(orc_sim* s, obj_t* o, double wx, double wy, double wz, double tx, double ty, double tz) {
  const double b = 0.5;
  double l0 = b * sin(ORC_PI / 3.0) * 2. / 3.;
  for (int i = 0; i < o->len; ++i) {
    double* p0 = BP(s, o, 0, i);
    double* p1 = BP(s, o, 1, i);
    double* p2 = BP(s, o, 2, i);
    p0[0] = 0.0;
    p0[1] = 0.0;
    p0[2] = b * i;
    p0[0] -= l0;
    p1[2] = b * i;
    p1[1] = b / 2.0;
    p1[0] = b * sin(ORC_PI / 3.0) - l0;
    p2[2] = b * i;
    p2[1] = -b / 2.0;
    p2[0] = b * sin(ORC_PI / 3.0) - l0;
  }
  for (int j = 0; j < o->rods; ++j)
    for (int i = 0; i < o->len; ++i) {
      double* p = BP(s, o, j, i);
      double xi = p[0], yi = p[1], zi = p[2];
      p[0] = zi * sin(ty) + cos(ty) * (xi * cos(tz) - yi * sin(tz));
      p[1] = cos(tx) * (yi * cos(tz) + xi * sin(tz)) -
             sin(tx) * (zi * cos(ty) + sin(ty) * (-(xi * cos(tz)) + yi * sin(tz)));
      p[2] = sin(tx) * (yi * cos(tz) + xi * sin(tz)) +
             cos(tx) * (zi * cos(ty) + sin(ty) * (-(xi * cos(tz)) + yi * sin(tz)));
    }
  for (int i = 0; i < o->rods; ++i)
    for (int j = 0; j < o->len; ++j) {
      double* p = BP(s, o, i, j);
      p[0] += wx;
      p[1] += wy;
      p[2] += wz;
    }
}

int orc_add_cilia(orc_sim* s, int kind, int rodlength, double beatstrength, double bending,
                  double min_bend, double max_bend, double m_speed, double k, double x, double y,
                  double z, double thetax, double thetay, double thetaz, int startidx, int num_anker,
                  double power_dur, double recovery_dur, double start_delay) {
  if (rodlength < 2) return -1;
  obj_t* o = new_obj(s, kind == 1 ? OBJ_CBCILIA : OBJ_CILIA, 3, rodlength);
  o->beatstrength = beatstrength;
  o->bending = bending;
  o->min_bend = min_bend;
  o->max_bend = max_bend;
  o->m_speed = m_speed;
  o->k = k;
  o->startidx = startidx;
  o->num_anker = num_anker;
  o->start = num_anker; /* cilia.cpp:100,107 */
  o->midpnt = o->start;
  o->newlength = (double*)malloc((size_t)rodlength * sizeof(double));
  o->oldlength = (double*)malloc((size_t)rodlength * sizeof(double));
  for (int i = 0; i < rodlength; ++i) o->newlength[i] = o->oldlength[i] = 0.5;
  o->power_dur = power_dur;
  o->recovery_dur = recovery_dur;
  o->tstroke = kind == 1 ? start_delay : 0.0; /* ConstantBeatCilia.h:18-20 */
  cilia_create(s, o, x, y, z, thetax, thetay, thetaz);
  return s->nobj - 1;
}

/* Matrix<double,2>::get_closest_idx (src/libcilia/Matrix.h:602-615) */
static int closest_sphere_bead(orc_sim* s, const obj_t* sp, const double* p) {
  double min_dist = 9999;
  int min_idx = 0;
  for (int i = 0; i < sp->len; ++i) {
    double d = sqdist3(BP(s, sp, 0, i), p);
    if (min_dist > d) {
      min_dist = d;
      min_idx = i;
    }
  }
  return min_idx;
}

/* Clami::add_springs_for_rods_idx (src/clami.cpp:152-174): nearest sphere bead
 * and its neighbours 1..count-1 (the last listed neighbour is not attached). */
static void clami_attach(orc_sim* s, obj_t* cl, int sphere_obj, int cil_obj, int wo) {
  for (int j = 0; j < 3; ++j) {
    obj_t* sp = &s->objs[sphere_obj];
    obj_t* ci = &s->objs[cil_obj];
    const double* pc = BP(s, ci, j, wo);
    int idx = closest_sphere_bead(s, sp, pc);
    int cnt = sp->neilist[idx][0];
    cl->springs = (attach_t*)realloc(cl->springs, (size_t)(cl->nspr + cnt + 1) * sizeof(attach_t));
    attach_t* a = &cl->springs[cl->nspr++];
    a->cil_obj = cil_obj;
    a->sphere_bead = idx;
    a->rod = j;
    a->bead = wo;
    a->l0 = sqrt(sqdist3(BP(s, sp, 0, idx), pc));
    for (int n = 1; n < cnt; ++n) {
      int sb = sp->neilist[idx][n];
      attach_t* b = &cl->springs[cl->nspr++];
      b->cil_obj = cil_obj;
      b->sphere_bead = sb;
      b->rod = j;
      b->bead = wo;
      b->l0 = sqrt(sqdist3(BP(s, sp, 0, sb), pc));
    }
  }
}

/* Clami::Clami + create_cilia + init_attachment_springs (src/clami.cpp:32-184) */
int orc_add_clami(orc_sim* s, double radius, double k, double x, double y, double z, int nrings,
                  const int* num_eq, const double* y_thetas_deg, const double* theta_offset,
                  const double* start_delays, int cil_kind, int rodlength, double beatstrength,
                  double bending, double min_bend, double max_bend, double m_speed, double cil_k,
                  double thetaz, double power_dur, double recovery_dur) {
  if (radius <= 0.0) return -1;
  int sph = orc_add_sphere(s, radius, k, x, y, z, 643);
  int ncil = 0;
  for (int i = 0; i < nrings; ++i) ncil += num_eq[i];
  int* cils = (int*)malloc((size_t)(ncil > 0 ? ncil : 1) * sizeof(int));
  attach_t* springs = NULL;
  int nspr = 0;
  obj_t tmp;
  memset(&tmp, 0, sizeof tmp);
  int ci = 0;
  for (int i = 0; i < nrings; ++i) {
    double thetaY = y_thetas_deg[i];
    thetaY *= ORC_PI / 180.;
    double off = theta_offset[i];
    int nx = num_eq[i];
    for (int j = 0; j < nx; ++j) {
      double thetaX = off + 2 * ORC_PI * j / nx;
      double delay = start_delays ? start_delays[ci] : 0.0;
      const int wo = 3;
      double r = s->objs[sph].radius - wo * 0.5;
      double pc[3] = {r * sin(thetaY), -r * cos(thetaY) * sin(thetaX), r * cos(thetaX) * cos(thetaY)};
      pc[0] += x;
      pc[1] += y;
      pc[2] += z;
      int co = orc_add_cilia(s, cil_kind, rodlength, beatstrength, bending, min_bend, max_bend, m_speed,
                             cil_k, pc[0], pc[1], pc[2], thetaX, thetaY, thetaz, 0, 2, power_dur,
                             recovery_dur, delay);
      cils[ci++] = co;
      tmp.springs = springs;
      tmp.nspr = nspr;
      int wod = (int)(wo * 0.5 / 0.5);
      clami_attach(s, &tmp, sph, co, 0);
      clami_attach(s, &tmp, sph, co, wod);
      springs = tmp.springs;
      nspr = tmp.nspr;
    }
  }
  obj_t* cl = new_obj(s, OBJ_CLAMI, 0, 0);
  cl->k = k;
  cl->sphere_obj = sph;
  cl->ncil = ncil;
  cl->cil_objs = cils;
  cl->springs = springs;
  cl->nspr = nspr;
  return s->nobj - 1;
}

int orc_num_objects(const orc_sim* s) { return s->nobj; }
void orc_object_info(const orc_sim* s, int obj, int* info5) {
  const obj_t* o = &s->objs[obj];
  info5[0] = o->kind;
  info5[1] = o->rods;
  info5[2] = o->len;
  info5[3] = o->startidx;
  info5[4] = (int)o->boff;
}
long orc_bead_count(const orc_sim* s) { return s->nb; }
void orc_beads_get(const orc_sim* s, double* pos, double* vel) {
  if (pos) memcpy(pos, s->bpos, 3 * (size_t)s->nb * sizeof(double));
  if (vel) memcpy(vel, s->bvel, 3 * (size_t)s->nb * sizeof(double));
}
int orc_beads_set(orc_sim* s, const double* pos, const double* vel) {
  if (pos) memcpy(s->bpos, pos, 3 * (size_t)s->nb * sizeof(double));
  if (vel) memcpy(s->bvel, vel, 3 * (size_t)s->nb * sizeof(double));
  return 0;
}
int orc_cilium_state(const orc_sim* s, int obj, double* out) {
  const obj_t* o = &s->objs[obj];
  if (o->kind != OBJ_CILIA && o->kind != OBJ_CBCILIA) return -1;
  for (int i = 0; i < o->len; ++i) {
    out[i] = o->newlength[i];
    out[o->len + i] = o->oldlength[i];
  }
  out[2 * o->len] = o->midpnt;
  out[2 * o->len + 1] = o->tstroke;
  return 0;
}
double orc_sphere_headbond(const orc_sim* s, int obj) { return s->objs[obj].headbond; }
int orc_clami_springs(const orc_sim* s, int obj, double* out, int max_rows) {
  const obj_t* o = &s->objs[obj];
  if (o->kind != OBJ_CLAMI) return -1;
  int n = o->nspr < max_rows ? o->nspr : max_rows;
  for (int i = 0; i < n; ++i) {
    out[5 * i + 0] = o->springs[i].cil_obj;
    out[5 * i + 1] = o->springs[i].sphere_bead;
    out[5 * i + 2] = o->springs[i].rod;
    out[5 * i + 3] = o->springs[i].bead;
    out[5 * i + 4] = o->springs[i].l0;
  }
  return o->nspr;
}

/* -------------------------------------------------------------- binning -- */
/* MPCD::box (src/libcilia/mpcd.cpp:130-138), anull = 1 */
static inline int cell_index(const orc_sim* s, const double* p) {
  double r = 0.0, stride = 1.0;
  for (int q = 0; q < 3; ++q) {
    double xa = p[q] + s->a[q];
    double f = floor(xa) - floor(xa / s->L[q]) * s->L[q];
    r += stride * f;
    stride *= s->L[q];
  }
  return (int)r;
}

/* add_impuls for every fluid particle then every movable bead, in that order
 * (src/libcilia/fluid.cpp:152-167, src/libcilia/mdobject.cpp:62-72). */
static void rebin(orc_sim* s) {
  long tot = s->n + s->nb;
  s->cell_of = (int*)realloc(s->cell_of, (size_t)(tot > 0 ? tot : 1) * sizeof(int));
  s->members = (long*)realloc(s->members, (size_t)(tot > 0 ? tot : 1) * sizeof(long));
  memset(s->cstart, 0, (size_t)(s->ncell + 1) * sizeof(long));
#pragma omp parallel for schedule(static) num_threads(s->threads) if (s->threads > 1)
  for (long i = 0; i < s->n; ++i) s->cell_of[i] = cell_index(s, s->pos + 3 * i);
  for (long b = 0; b < s->nb; ++b)
    s->cell_of[s->n + b] = s->bmass[b] > 0.0 ? cell_index(s, s->bpos + 3 * b) : -1;
  for (long i = 0; i < tot; ++i)
    if (s->cell_of[i] >= 0) s->cstart[s->cell_of[i] + 1]++;
  for (long c = 0; c < s->ncell; ++c) s->cstart[c + 1] += s->cstart[c];
  long* fill = (long*)malloc((size_t)s->ncell * sizeof(long));
  memcpy(fill, s->cstart, (size_t)s->ncell * sizeof(long));
  for (long i = 0; i < tot; ++i)
    if (s->cell_of[i] >= 0) s->members[fill[s->cell_of[i]]++] = i;
  free(fill);
}

void orc_init_bins(orc_sim* s) {
  for (int k = 0; k < s->nobj; ++k) { /* MDObject::init (mdobject.cpp:153-160) */
    obj_t* o = &s->objs[k];
    for (int r = 0; r < o->rods; ++r)
      for (int j = 0; j < o->len; ++j) s->bmass[o->boff + (long)r * o->len + j] = j >= o->startidx ? 5.0 : 0.0;
  }
  rebin(s);
}

/* ------------------------------------------------------------ collision -- */
static inline double* vel_of(orc_sim* s, long m, double* mass) {
  if (m < s->n) {
    *mass = 1.0;
    return s->vel + 3 * m;
  }
  *mass = s->bmass[m - s->n];
  return s->bvel + 3 * (m - s->n);
}

/* MPCD::next_tstep for one cell (src/libcilia/mpcd.cpp:149-246) with the
 * rotation matrix of generate_collision_matrix (mpcd.cpp:269-295). */
static int collide_cell(orc_sim* s, long cid, mt_t* g, const double* inj_gamma, const double* inj_axis,
                        const double* inj_virt, double* rec_gamma, double* rec_axis, double* rec_virt) {
  const double calpha = -0.6427876, salpha = 0.76604444; /* mpcd.h:74-75 */
  double ux = 0.0, uy = 0.0, uz = 0.0, le = 0.0;
  int num = 0, masse = 0;
  long b0 = s->cstart[cid], b1 = s->cstart[cid + 1];
  for (long m = b0; m < b1; ++m) {
    double pm;
    double* v = vel_of(s, s->members[m], &pm);
    ux += v[0] * pm;
    uy += v[1] * pm;
    uz += v[2] * pm;
    masse += (int)pm;
    le += pm * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  }
  num = (int)(b1 - b0);
  int err = 0;
  if (num > 0) {
    /* wall layers: virtual particles fill a cell up to rho = 10 with momentum
       N(0, sqrt(dm kT)) per component, drawn before the cell's Gamma variate
       (src/libcilia/mpcd.cpp:175-198; the top-layer test is a strict `>`, so
       the first top-layer cell takes none) */
    const long layer = (long)s->L[0] * s->L[1];
    if (s->walls && (cid < layer || cid > layer * (s->L[2] - 1)) && num < 10) {
      const int dm = 10 - num;
      double pv[3];
      for (int q = 0; q < 3; ++q) pv[q] = inj_virt ? inj_virt[3 * cid + q] : sqrt((double)dm * 1.0) * mt_normal(g);
      if (rec_virt)
        for (int q = 0; q < 3; ++q) rec_virt[3 * cid + q] = pv[q];
      ux += pv[0];
      uy += pv[1];
      uz += pv[2];
      masse += dm;
      num += dm;
      le += (pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]) / dm;
    }
    ux /= masse;
    uy /= masse;
    uz /= masse;
    double rel = le - (ux * ux + uy * uy + uz * uz) * masse;
    double sc = 1.0;
    double gam = -1.0;
    if (rel > 0 && num > 1) {
      if (inj_gamma) {
        gam = inj_gamma[cid];
        if (gam < 0) err = 1;
      } else {
        gam = mt_gamma(g, num);
      }
      sc = sqrt(gam / (rel * 0.5));
    }
    double rx, ry, rz;
    if (inj_axis) {
      rx = inj_axis[3 * cid + 0];
      ry = inj_axis[3 * cid + 1];
      rz = inj_axis[3 * cid + 2];
    } else {
      double phi = 2 * ORC_PI * mt_rand(g);
      double theta = 2.0 * mt_rand(g) - 1.0;
      double s1 = sqrt(1.0 - theta * theta);
      rx = s1 * cos(phi);
      ry = s1 * sin(phi);
      rz = theta;
    }
    if (rec_gamma) rec_gamma[cid] = gam;
    if (rec_axis) {
      rec_axis[3 * cid + 0] = rx;
      rec_axis[3 * cid + 1] = ry;
      rec_axis[3 * cid + 2] = rz;
    }
    double R[3][3];
    R[0][0] = rx * rx + (1.0 - rx * rx) * calpha;
    R[0][1] = rx * ry * (1.0 - calpha) - rz * salpha;
    R[0][2] = rx * rz * (1.0 - calpha) + ry * salpha;
    R[1][0] = rx * ry * (1.0 - calpha) + rz * salpha;
    R[1][1] = ry * ry + (1.0 - ry * ry) * calpha;
    R[1][2] = ry * rz * (1.0 - calpha) - rx * salpha;
    R[2][0] = rx * rz * (1.0 - calpha) - ry * salpha;
    R[2][1] = ry * rz * (1.0 - calpha) + rx * salpha;
    R[2][2] = rz * rz + (1.0 - rz * rz) * calpha;
    for (long m = b0; m < b1; ++m) {
      double pm;
      double* v = vel_of(s, s->members[m], &pm);
      double w0 = v[0] - ux, w1 = v[1] - uy, w2 = v[2] - uz;
      v[0] = ux + (R[0][0] * w0 + R[0][1] * w1 + R[0][2] * w2) * sc;
      v[1] = uy + (R[1][0] * w0 + R[1][1] * w1 + R[1][2] * w2) * sc;
      v[2] = uz + (R[2][0] * w0 + R[2][1] * w1 + R[2][2] * w2) * sc;
      le -= pm * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
  } else {
    if (rec_gamma) rec_gamma[cid] = -2.0;
  }
  s->l_energy[cid] = le;
  return err;
}

static int collide(orc_sim* s, const double* inj_gamma, const double* inj_axis, const double* inj_virt,
                   double* rec_gamma, double* rec_axis, double* rec_virt) {
  int err = 0;
  if (s->threads <= 1) {
    for (long c = 0; c < s->ncell; ++c)
      err |= collide_cell(s, c, &s->rng, inj_gamma, inj_axis, inj_virt, rec_gamma, rec_axis, rec_virt);
  } else {
#pragma omp parallel num_threads(s->threads) reduction(| : err)
    {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
#pragma omp for schedule(static)
      for (long c = 0; c < s->ncell; ++c)
        err |= collide_cell(s, c, &s->trng[tid], inj_gamma, inj_axis, inj_virt, rec_gamma, rec_axis, rec_virt);
    }
  }
  long double tot = 0.0L;
  for (long c = 0; c < s->ncell; ++c) tot += s->l_energy[c]; /* mpcd.cpp:243-246 */
  s->diss += tot;
  return err;
}

/* ------------------------------------------------------------------- MD -- */
/* MDObject::spring, one-sided (src/libcilia/mdobject.cpp:8-17) */
static inline void spring1(double* f, const double* p1, const double* p0, double b, double k) {
  double fac = -2.0 * k * (1.0 - b / sqrt(sqdist3(p1, p0)));
  f[0] += (p1[0] - p0[0]) * fac;
  f[1] += (p1[1] - p0[1]) * fac;
  f[2] += (p1[2] - p0[2]) * fac;
}

/* Cilia::length (src/cilia.cpp:79-121): active rest length of bond i */
static double cilia_length(orc_sim* s, obj_t* o, int i) {
  const double bondlength = 0.5;
  double l = bondlength;
  double tl = sqrt(sqdist3(BP(s, o, 0, i), BP(s, o, 0, i + 1)));
  if (i < o->midpnt - 2.0) {
    l = bondlength + o->beatstrength *
                         pow(1.0 - (i - o->num_anker - 1.0) / (o->len - o->num_anker - 1.0), 2.5) * 0.5 *
                         (1.0 - 1.0 / (o->midpnt - i - 1.0));
  } else {
    l = bondlength - 2.0 * o->beatstrength / (pow((i - o->midpnt), 2.0) + 1.0);
  }
  if (fabs(l - tl) > o->bending) {
    tl = tl + o->bending - 2.0 * o->bending * (l < tl);
    if (((l - o->oldlength[i]) * (tl - o->oldlength[i])) > 0) {
      l = tl;
    } else {
      l = o->oldlength[i];
    }
  }
  return l;
}

#define SP(i, j, b, k) spring1(F(i), P(i), P(j), b, k)
/* Cilia::recalcforce + addcross (src/cilia.cpp:127-239); bead index
 * rod*len + bead as get_row_by_idx (Matrix.h:716) */
static void cilia_forces(orc_sim* s, obj_t* o) {
  const double bondlength = 0.5, crosslength = sqrt(2.0) * 0.5, cs = 1.0;
  const int R = o->len;
  const double k = o->k;
  double* base_p = s->bpos + 3 * o->boff;
  double* base_f = s->bfrc + 3 * o->boff;
#define P(i) (base_p + 3 * (long)(i))
#define F(i) (base_f + 3 * (long)(i))
  if (fmod(s->globalt + s->ststep / 10., 0.01) < s->ststep) {
    for (int i = o->num_anker - 1; i < R - 1; ++i) {
      o->newlength[i] = cilia_length(s, o, i);
      o->oldlength[i] = o->newlength[i];
    }
  }
  memset(base_f, 0, 3 * (size_t)o->rods * R * sizeof(double));
  for (int i = 0; i < R - 1; i++) {
    SP(i, i + 1, o->newlength[i], k);
    SP(i + 1, i, o->newlength[i], k);
    SP(R + i, R + i + 1, bondlength, k);
    SP(R + i + 1, R + i, bondlength, k);
    SP(2 * R + i, 2 * R + i + 1, bondlength, k);
    SP(2 * R + i + 1, 2 * R + i, bondlength, k);
  }
  for (int i = 0; i < R; ++i) {
    SP(i, i + R, bondlength, k);
    SP(i, i + 2 * R, bondlength, k);
    SP(i + R, i, bondlength, k);
    SP(i + R, i + 2 * R, bondlength, k);
    SP(i + 2 * R, i, bondlength, k);
    SP(i + 2 * R, i + R, bondlength, k);
  }
  for (int i = 0; i < R - 1; ++i) {
    double li = sqrt(bondlength * bondlength + bondlength * o->newlength[i]);
    SP(i, i + R + 1, li, cs * k);
    SP(i, i + 2 * R + 1, li, cs * k);
    SP(i + R, i + 1, li, cs * k);
    SP(i + 2 * R, i + 1, li, cs * k);
    SP(i + R, i + 2 * R + 1, crosslength, cs * k);
    SP(i + 2 * R, i + R + 1, crosslength, cs * k);
  }
  for (int i = 1; i < R; ++i) {
    double li = sqrt(bondlength * bondlength + bondlength * o->newlength[i - 1]);
    SP(i, i + R - 1, li, cs * k);
    SP(i, i + 2 * R - 1, li, cs * k);
    SP(i + R, i - 1, li, cs * k);
    SP(i + 2 * R, i - 1, li, cs * k);
    SP(i + R, i + 2 * R - 1, crosslength, cs * k);
    SP(i + 2 * R, i + R - 1, crosslength, cs * k);
  }
#undef P
#undef F
}

/* Sphere::recalcforce (src/sphere.cpp:87-119): accumulates, no reset */
static void sphere_forces(orc_sim* s, obj_t* o) {
  double* base_p = s->bpos + 3 * o->boff;
  double* base_f = s->bfrc + 3 * o->boff;
#define P(i) (base_p + 3 * (long)(i))
#define F(i) (base_f + 3 * (long)(i))
  for (int i = 1; i < o->npart; i++) {
    SP(0, i, o->radius, 0.1 * o->k);
    SP(i, 0, o->radius, 0.1 * o->k);
  }
  for (int i = 1; i < o->npart; i++)
    for (int j = 1; j < o->neilist[i][0] + 1; j++) SP(i, o->neilist[i][j], o->headbond, o->k);
#undef P
#undef F
}
#undef SP

/* Clami::global_forces (src/clami.cpp:188-198), vector spring (mdobject.cpp:19-29) */
static void clami_forces(orc_sim* s, obj_t* cl) {
  obj_t* sp = &s->objs[cl->sphere_obj];
  for (int i = 0; i < cl->nspr; ++i) {
    attach_t* a = &cl->springs[i];
    obj_t* ci = &s->objs[a->cil_obj];
    double* p0 = BP(s, sp, 0, a->sphere_bead);
    double* p1 = BP(s, ci, a->rod, a->bead);
    double f[3] = {0., 0., 0.};
    double d = sqrt(sqdist3(p0, p1));
    if (d != 0) {
      double fac = -2.0 * cl->k * (1.0 - a->l0 / d);
      for (int q = 0; q < 3; ++q) f[q] = (p0[q] - p1[q]) * fac;
    }
    double* f0 = BF(s, sp, 0, a->sphere_bead);
    double* f1 = BF(s, ci, a->rod, a->bead);
    for (int q = 0; q < 3; ++q) f0[q] += f[q];
    for (int q = 0; q < 3; ++q) f1[q] -= f[q];
  }
}

/* GlobalForces::recalc_forces and vdw_force with -DREPELLING=eps
 * (src/libcilia/globalforces.cpp:22-95, constants src/libcilia/globalforces.h:22-28:
 * cutoff 1.5, N = 4).  The reference's code indexes a `cilias` list that
 * GlobalForces does not declare, so its -DREPELLING build does not compile;
 * restated here over the cilia in object order.  For every pair i < j (j from
 * the last down) whose bounding boxes of section centroids (min from 999999,
 * max from 0, as Cilia::getBoundingBox, src/cilia.cpp:435-465) overlap within
 * the cutoff, every filament-0 bead pair (k, l) on the stride-N lattices
 * k = 1 + N/2, 1 + N/2 + N, ... and l = len_j - 1 - N/2, ... down to l >= k,
 * closer than N * cutoff, adds for sections kk = k - N/2 .. k + N/2 - 1 and
 * ll = l + N/2 down to max(l - N/2, kk) the harmonic repulsion of the section
 * centroids, F = -2 eps (1 - cutoff / |d|) d for |d| < cutoff, to all three
 * filaments of section kk and its negative to those of ll.  Sections past a
 * cilium's end (k + 1 = len, which the reference reads beyond its array) are
 * skipped. */
static void centroid(orc_sim* s, const obj_t* o, int j, double* c) {
  c[0] = c[1] = c[2] = 0.0;
  for (int r = 0; r < o->rods; ++r) {
    const double* p = BP(s, o, r, j);
    c[0] += p[0];
    c[1] += p[1];
    c[2] += p[2];
  }
}

static void cilia_bbox(orc_sim* s, const obj_t* o, double* mn, double* mx) {
  for (int q = 0; q < 3; ++q) {
    mn[q] = 999999.0;
    mx[q] = 0.0;
  }
  for (int j = 0; j < o->len; ++j) {
    double c[3];
    centroid(s, o, j, c);
    for (int q = 0; q < 3; ++q) {
      const double a = c[q] / o->rods;
      if (a > mx[q]) mx[q] = a;
      if (a < mn[q]) mn[q] = a;
    }
  }
}

static void repel_pair(orc_sim* s, obj_t* ci, obj_t* cj, int k, int l) {
  const int N = 4;
  const double cutoff = 1.5, eps = s->repelling;
  for (int kk = k - N / 2; kk < k + N / 2; ++kk) {
    if (kk >= ci->len) break;
    double x0[3];
    centroid(s, ci, kk, x0);
    for (int ll = l + N / 2; ll >= l - N / 2 && ll >= kk; --ll) {
      double x1[3], d[3];
      centroid(s, cj, ll, x1);
      for (int q = 0; q < 3; ++q) d[q] = (x0[q] - x1[q]) / 3.0;
      const double dis = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      if (!(dis < cutoff)) continue;
      s->contacts++;
      const double force = -2.0 * eps * (1.0 - cutoff / dis);
      for (int r = 0; r < ci->rods; ++r) {
        double* f = BF(s, ci, r, kk);
        for (int q = 0; q < 3; ++q) f[q] += d[q] * force;
      }
      for (int r = 0; r < cj->rods; ++r) {
        double* f = BF(s, cj, r, ll);
        for (int q = 0; q < 3; ++q) f[q] -= d[q] * force;
      }
    }
  }
}

static void repel_forces(orc_sim* s) {
  const int N = 4;
  const double cutoff = 1.5;
  for (int i = 0; i < s->nobj; ++i) {
    obj_t* ci = &s->objs[i];
    if (ci->kind != OBJ_CILIA && ci->kind != OBJ_CBCILIA) continue;
    double mn1[3], mx1[3];
    cilia_bbox(s, ci, mn1, mx1);
    for (int j = s->nobj - 1; j > i; --j) {
      obj_t* cj = &s->objs[j];
      if (cj->kind != OBJ_CILIA && cj->kind != OBJ_CBCILIA) continue;
      double mn2[3], mx2[3];
      cilia_bbox(s, cj, mn2, mx2);
      int overlap = 1;
      for (int q = 0; q < 3; ++q)
        overlap &= (mn2[q] - mx1[q] < cutoff) && (mn1[q] - mx2[q] < cutoff);
      if (!overlap) continue;
      for (int k = 1 + N / 2; k < ci->len; k += N)
        for (int l = cj->len - 1 - N / 2; l >= k; l -= N)
          if (sqrt(sqdist3(BP(s, ci, 0, k), BP(s, cj, 0, l))) < N * cutoff) repel_pair(s, ci, cj, k, l);
    }
  }
}

void orc_set_repelling(orc_sim* s, double eps) {
  s->repelling = eps;
  s->contacts = 0;
}
long orc_contacts(const orc_sim* s) { return s->contacts; }

/* Simulation::recalc_forces (src/simulation.cpp:202-215) */
static void recalc_forces(orc_sim* s) {
  for (int k = 0; k < s->nobj; ++k) {
    obj_t* o = &s->objs[k];
    if (o->kind == OBJ_CILIA || o->kind == OBJ_CBCILIA) cilia_forces(s, o);
    else if (o->kind == OBJ_SPHERE) sphere_forces(s, o);
  }
  if (s->repelling != 0.0) repel_forces(s);
  for (int k = 0; k < s->nobj; ++k)
    if (s->objs[k].kind == OBJ_CLAMI) clami_forces(s, &s->objs[k]);
}

/* md_loop_start / md_loop (src/libcilia/mdobject.cpp:36-60) */
static void md_kick_drift(orc_sim* s, double kick) {
  for (int k = 0; k < s->nobj; ++k) {
    obj_t* o = &s->objs[k];
    for (int r = 0; r < o->rods; ++r)
      for (int j = o->startidx; j < o->len; ++j) {
        double *v = BV(s, o, r, j), *x = BP(s, o, r, j), *f = BF(s, o, r, j);
        for (int q = 0; q < 3; ++q) v[q] += f[q] * kick;
        for (int q = 0; q < 3; ++q) x[q] += v[q] * s->ststep;
        f[0] = f[1] = f[2] = 0.0;
      }
  }
}

/* md_loop_stop (src/libcilia/mdobject.cpp:62-72) without the binning */
static void md_half_kick(orc_sim* s) {
  for (int k = 0; k < s->nobj; ++k) {
    obj_t* o = &s->objs[k];
    for (int r = 0; r < o->rods; ++r)
      for (int j = o->startidx; j < o->len; ++j) {
        double *v = BV(s, o, r, j), *f = BF(s, o, r, j);
        for (int q = 0; q < 3; ++q) v[q] += f[q] * (s->ststep / 2.0);
        f[0] = f[1] = f[2] = 0.0;
      }
  }
}

/* Cilia::localbend (src/cilia.cpp:68-77) */
static double cilia_localbend(orc_sim* s, obj_t* o, int a, int b) {
  double l = 0;
  for (int i = a; i < b - 1; i++) {
    l += 2.0 * sqrt(sqdist3(BP(s, o, 0, i), BP(s, o, 0, i + 1)));
    l -= sqrt(sqdist3(BP(s, o, 1, i), BP(s, o, 1, i + 1)));
    l -= sqrt(sqdist3(BP(s, o, 2, i), BP(s, o, 2, i + 1)));
  }
  return l;
}

/* Cilia::switch_logic (src/cilia.cpp:241-258) and
 * ConstantBeatCilia::switch_logic (src/ConstantBeatCilia.cpp:8-23) */
static void switch_logic(orc_sim* s) {
  for (int k = 0; k < s->nobj; ++k) {
    obj_t* o = &s->objs[k];
    if (o->kind == OBJ_CBCILIA) {
      if (s->globalt - o->tstroke >= o->power_dur && o->midpnt == o->start) o->midpnt += 1;
      if (s->globalt - o->tstroke - o->power_dur >= o->recovery_dur && o->midpnt > o->start) {
        o->tstroke = s->globalt;
        o->midpnt = o->start;
      }
      if (o->midpnt > o->start) o->midpnt += s->tstep / o->m_speed;
    } else if (o->kind == OBJ_CILIA) {
      if ((o->midpnt == o->start) && s->globalt - o->tstroke > 100.0) o->midpnt += 1;
      if ((cilia_localbend(s, o, 0, o->len) > o->max_bend) && (o->midpnt > o->start)) {
        o->tstroke = s->globalt;
        o->midpnt = o->start;
      }
      if (o->midpnt > o->start) o->midpnt += s->tstep / o->m_speed;
    }
  }
}

/* ----------------------------------------------------------------- step -- */
/* MPCD::move (src/libcilia/mpcd.cpp:340-376): streaming, then bounce-back at
 * the walls (vwx = vwy = 0); Fluid::move's body force (fluid.cpp:156-158) */
static void stream_fluid(orc_sim* s) {
  const double ztop = (double)(s->L[2] - 1);
  const double kick = s->gravity != 0.0 ? s->gravity * cos(s->globalt * s->omega) * s->tstep : 0.0;
#pragma omp parallel for schedule(static) num_threads(s->threads) if (s->threads > 1)
  for (long i = 0; i < s->n; ++i) {
    double* x = s->pos + 3 * i;
    double* v = s->vel + 3 * i;
    for (int q = 0; q < 3; ++q) x[q] += v[q] * s->tstep;
    if (s->walls) {
      if (x[2] > ztop) {
        if (s->walls == 1) {
          const double t2 = (x[2] - ztop) / v[2];
          v[0] = -v[0];
          v[1] = -v[1];
          v[2] = -v[2];
          x[0] += 2.0 * t2 * v[0];
          x[1] += 2.0 * t2 * v[1];
          x[2] += 2.0 * t2 * v[2];
        } else {
          v[2] = -v[2];
          x[2] = -x[2] + ztop * 2.0;
        }
      }
      if (x[2] < 0) {
        const double t2 = x[2] / v[2];
        v[0] = -v[0];
        v[1] = -v[1];
        v[2] = -v[2];
        x[0] += v[0] * 2.0 * t2;
        x[1] += v[1] * 2.0 * t2;
        x[2] += v[2] * 2.0 * t2;
      }
    }
    if (kick != 0.0) v[0] += kick;
  }
}

void orc_set_walls(orc_sim* s, int walls) { s->walls = walls; }
void orc_set_gravity(orc_sim* s, double g, double omega) {
  s->gravity = g;
  s->omega = omega;
}

/* Simulation::next_tstep (src/simulation.cpp:217-265) */
int orc_step(orc_sim* s, const double* inj_shift_next, const double* inj_gamma, const double* inj_axis,
             double* rec_shift_next, double* rec_gamma, double* rec_axis) {
  return orc_step_walls(s, inj_shift_next, inj_gamma, inj_axis, NULL, rec_shift_next, rec_gamma, rec_axis, NULL);
}

int orc_step_walls(orc_sim* s, const double* inj_shift_next, const double* inj_gamma, const double* inj_axis,
                   const double* inj_virt, double* rec_shift_next, double* rec_gamma, double* rec_axis,
                   double* rec_virt) {
  const int n = (int)((s->tstep + 0.00000001) / s->ststep);
  int err = collide(s, inj_gamma, inj_axis, inj_virt, rec_gamma, rec_axis, rec_virt);
  if (s->nb > 0) {
    recalc_forces(s);
    md_kick_drift(s, s->ststep / 2.0);
    recalc_forces(s);
    for (int k = 1; k < n; k++) {
      s->globalt += s->ststep;
      md_kick_drift(s, s->ststep);
      recalc_forces(s);
    }
  } else {
    for (int k = 1; k < n; k++) s->globalt += s->ststep;
  }
  s->globalt += s->ststep;
  if (inj_shift_next) {
    memcpy(s->a, inj_shift_next, sizeof s->a);
  } else {
    for (int q = 0; q < 3; ++q) s->a[q] = mt_dblexc(&s->rng); /* mpcd.cpp:249-253 */
  }
  if (rec_shift_next) memcpy(rec_shift_next, s->a, sizeof s->a);
  stream_fluid(s);
  if (s->nb > 0) md_half_kick(s);
  rebin(s);
  switch_logic(s);
  return err;
}

double orc_diss_energy(const orc_sim* s) { return (double)s->diss; }
void orc_reset_diss(orc_sim* s) { s->diss = 0.0L; }

void orc_set_threads(orc_sim* s, int threads) {
  if (threads < 1) threads = 1;
  s->threads = threads;
  free(s->trng);
  s->trng = (mt_t*)malloc((size_t)threads * sizeof(mt_t));
  for (int t = 0; t < threads; ++t) mt_seed(&s->trng[t], mt_u32(&s->rng) + (uint32_t)t);
}

/* MPCD::debug totals (src/libcilia/mpcd.cpp:404-467) */
void orc_observables(const orc_sim* s, double* out6) {
  double ux = 0, uy = 0, uz = 0, e = 0;
  long num = 0;
  double masse = 0;
  for (long i = 0; i < s->n; ++i) {
    const double* v = s->vel + 3 * i;
    ux += v[0];
    uy += v[1];
    uz += v[2];
    masse += 1.0;
    e += v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    num++;
  }
  for (long b = 0; b < s->nb; ++b) {
    double m = s->bmass[b];
    if (m <= 0) continue;
    const double* v = s->bvel + 3 * b;
    ux += v[0] * m;
    uy += v[1] * m;
    uz += v[2] * m;
    masse += m;
    e += m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    num++;
  }
  out6[0] = ux / masse;
  out6[1] = uy / masse;
  out6[2] = uz / masse;
  out6[3] = (double)num;
  out6[4] = masse;
  out6[5] = e / 3.0 / num;
}
