/*
 * oracle.c -- CPU FP64 restatement of the reference's collision / distance
 * path, used ONLY as test infrastructure: tests/, __graft_entry__.smoke() and
 * the cpu_baseline / --impl reference legs of bench.py call it as the checker.
 * Nothing on the product path links or calls this file.
 *
 * Every floating-point operation here is written out in the order the
 * reference (or, for the new sphere-arm scenes, the library's documented
 * semantics) performs it.  Build with -ffp-contract=off so that the compiler
 * never fuses a multiply and an add on its own; the only fused operations are
 * the explicit fma() calls that restate OpenBLAS ddot (np.linalg.norm).
 *
 * Reference files cited below are paths inside
 * src/multi_robot_multi_goal_planning/ of vhartman/multirobot-pathplanning-benchmark.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_ERR_ARG (-1)

/* ------------------------------------------------------------------------ */
/* numpy reductions                                                          */
/* ------------------------------------------------------------------------ */

/* np.sum of a contiguous float64 vector: numpy's pairwise summation
 * (8 partial accumulators for blocks up to 128, recursive halving above). */
static double np_pairwise_sum(const double *a, int64_t n) {
  if (n < 8) {
    double res = 0.0;
    for (int64_t i = 0; i < n; i++) res = res + a[i];
    return res;
  } else if (n <= 128) {
    double r[8];
    for (int j = 0; j < 8; j++) r[j] = a[j];
    int64_t i;
    for (i = 8; i < n - (n % 8); i += 8)
      for (int j = 0; j < 8; j++) r[j] = r[j] + a[i + j];
    double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    for (; i < n; i++) res = res + a[i];
    return res;
  } else {
    int64_t n2 = n / 2;
    n2 -= n2 % 8;
    return np_pairwise_sum(a, n2) + np_pairwise_sum(a + n2, n - n2);
  }
}

double orc_np_sum(const double *a, int64_t n) { return np_pairwise_sum(a, n); }

/* np.linalg.norm of a short float64 vector: sqrt(dot(x, x)) where OpenBLAS
 * ddot accumulates x_k*x_k with fused multiply-adds from 0 (dims <= 15). */
static double np_norm_sq(const double *x, int n) {
  double acc = 0.0;
  for (int k = 0; k < n; k++) acc = fma(x[k], x[k], acc);
  return acc;
}

/* ------------------------------------------------------------------------ */
/* generate_binary_search_indices  (problems/planning_env.py:34-51)          */
/* ------------------------------------------------------------------------ */
int orc_binary_indices(int64_t N, int64_t *out) {
  if (N <= 0) return ORC_OK;
  int64_t *qs = (int64_t *)malloc(sizeof(int64_t) * 2 * (size_t)N);
  if (!qs) return ORC_ERR_ARG;
  int64_t head = 0, tail = 0, idx = 0;
  qs[2 * tail] = 0; qs[2 * tail + 1] = N - 1; tail++;
  while (head < tail) {
    int64_t s = qs[2 * head], e = qs[2 * head + 1]; head++;
    int64_t mid = (s + e) / 2;   /* s,e >= 0: floor division */
    out[idx++] = mid;
    if (s <= mid - 1) { qs[2 * tail] = s; qs[2 * tail + 1] = mid - 1; tail++; }
    if (mid + 1 <= e) { qs[2 * tail] = mid + 1; qs[2 * tail + 1] = e; tail++; }
  }
  free(qs);
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Abstract point-agent scenes  (problems/abstract_env.py:41-109, 255-276)   */
/* ------------------------------------------------------------------------ */
typedef struct {
  int32_t n_agents, dim;
  int64_t *agent_off;   /* start of agent i's slice in q            */
  double *pair_thr;     /* [A*A]  agent_radii[i] + agent_radii[j]   */
  double *agent_r2;     /* [A]    agent_radii[i] ** 2               */
  int32_t n_boxes;
  double *box_lo, *box_hi; /* [n_boxes*dim] center -/+ bounds/2     */
  int32_t n_sph;
  double *sph_pos;      /* [n_sph*dim]                              */
  double *sph_thr;      /* [n_sph*A] obstacle radius + agent radius */
} orc_abstract;

void *orc_abstract_new(int32_t n_agents, int32_t dim, const int64_t *agent_off,
                       const double *pair_thr, const double *agent_r2,
                       int32_t n_boxes, const double *box_lo, const double *box_hi,
                       int32_t n_sph, const double *sph_pos, const double *sph_thr) {
  if (n_agents <= 0 || dim <= 0 || dim > 15) return NULL;
  orc_abstract *s = (orc_abstract *)calloc(1, sizeof(orc_abstract));
  s->n_agents = n_agents; s->dim = dim; s->n_boxes = n_boxes; s->n_sph = n_sph;
  s->agent_off = (int64_t *)malloc(sizeof(int64_t) * n_agents);
  memcpy(s->agent_off, agent_off, sizeof(int64_t) * n_agents);
  s->pair_thr = (double *)malloc(sizeof(double) * n_agents * n_agents);
  memcpy(s->pair_thr, pair_thr, sizeof(double) * n_agents * n_agents);
  s->agent_r2 = (double *)malloc(sizeof(double) * n_agents);
  memcpy(s->agent_r2, agent_r2, sizeof(double) * n_agents);
  size_t nb = (size_t)n_boxes * dim, ns = (size_t)n_sph * dim;
  s->box_lo = (double *)malloc(sizeof(double) * (nb + 1));
  s->box_hi = (double *)malloc(sizeof(double) * (nb + 1));
  if (nb) { memcpy(s->box_lo, box_lo, sizeof(double) * nb); memcpy(s->box_hi, box_hi, sizeof(double) * nb); }
  s->sph_pos = (double *)malloc(sizeof(double) * (ns + 1));
  s->sph_thr = (double *)malloc(sizeof(double) * ((size_t)n_sph * n_agents + 1));
  if (ns) {
    memcpy(s->sph_pos, sph_pos, sizeof(double) * ns);
    memcpy(s->sph_thr, sph_thr, sizeof(double) * (size_t)n_sph * n_agents);
  }
  return s;
}

void orc_abstract_free(void *p) {
  orc_abstract *s = (orc_abstract *)p;
  if (!s) return;
  free(s->agent_off); free(s->pair_thr); free(s->agent_r2); free(s->box_lo);
  free(s->box_hi); free(s->sph_pos); free(s->sph_thr); free(s);
}

/* Rectangle.collides_with_sphere (abstract_env.py:69-84):
 * closest = clip(c, min, max); sum((closest - c)**2) <= r**2 */
static int rect_hits(const double *lo, const double *hi, const double *c, int dim, double r2) {
  double sq[16];
  for (int k = 0; k < dim; k++) {
    double v = c[k] > lo[k] ? c[k] : lo[k];  /* np.maximum then np.minimum */
    v = v < hi[k] ? v : hi[k];
    double e = v - c[k];
    sq[k] = e * e;
  }
  return np_pairwise_sum(sq, dim) <= r2;
}

/* AbstractEnvironment.is_collision_free (abstract_env.py:255-276) */
int orc_abstract_config_free(const void *p, const double *q) {
  const orc_abstract *s = (const orc_abstract *)p;
  const int A = s->n_agents, dim = s->dim;
  double d[16];
  for (int i = 0; i < A; i++)
    for (int j = i + 1; j < A; j++) {
      const double *qi = q + s->agent_off[i], *qj = q + s->agent_off[j];
      for (int k = 0; k < dim; k++) d[k] = qi[k] - qj[k];
      if (sqrt(np_norm_sq(d, dim)) < s->pair_thr[i * A + j]) return 0;
    }
  for (int i = 0; i < A; i++) {
    const double *c = q + s->agent_off[i];
    for (int b = 0; b < s->n_boxes; b++)
      if (rect_hits(s->box_lo + (size_t)b * dim, s->box_hi + (size_t)b * dim, c, dim, s->agent_r2[i])) return 0;
    /* Sphere.collides_with_sphere (abstract_env.py:46-49) */
    for (int o = 0; o < s->n_sph; o++) {
      const double *pos = s->sph_pos + (size_t)o * dim;
      for (int k = 0; k < dim; k++) d[k] = pos[k] - c[k];
      if (sqrt(np_norm_sq(d, dim)) < s->sph_thr[(size_t)o * A + i]) return 0;
    }
  }
  return 1;
}

/* ------------------------------------------------------------------------ */
/* Deterministic FP64 sine/cosine used by the sphere-arm scenes.             */
/* Cody & Waite (1980) argument reduction by pi/2 with a three-part split    */
/* constant, then the Taylor series of sin and cos on [-pi/4, pi/4]          */
/* (coefficients (-1)^n/(2n+1)! and (-1)^n/(2n)!, correctly rounded),        */
/* evaluated by Horner's rule with separate multiplies and adds.  The GPU     */
/* library evaluates the identical sequence, so both sides agree bit for bit. */
/* ------------------------------------------------------------------------ */
static const double ORC_2_OVER_PI = 0x1.45f306dc9c883p-1;
static const double ORC_PIO2_1 = 0x1.921fb54400000p+0;
static const double ORC_PIO2_2 = 0x1.0b4611a600000p-34;
static const double ORC_PIO2_3 = 0x1.3198a2e037073p-69;
static const double ORC_S[9] = {-0x1.5555555555555p-3, 0x1.1111111111111p-7, -0x1.a01a01a01a01ap-13,
                                0x1.71de3a556c734p-19, -0x1.ae64567f544e4p-26, 0x1.6124613a86d09p-33,
                                -0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49, -0x1.2f49b46814157p-57};
static const double ORC_C[9] = {-0x1.0000000000000p-1, 0x1.5555555555555p-5, -0x1.6c16c16c16c17p-10,
                                0x1.a01a01a01a01ap-16, -0x1.27e4fb7789f5cp-22, 0x1.1eed8eff8d898p-29,
                                -0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-45, -0x1.6827863b97d97p-53};

void orc_sincos(double x, double *sn, double *cs) {
  if (!(fabs(x) < 0x1p30)) { *sn = NAN; *cs = NAN; return; }  /* non-finite or |x| >= 2^30 */
  double k = nearbyint(x * ORC_2_OVER_PI);
  double r = x - k * ORC_PIO2_1;
  r = r - k * ORC_PIO2_2;
  r = r - k * ORC_PIO2_3;
  double r2 = r * r;
  double ps = ORC_S[8];
  for (int i = 7; i >= 0; i--) ps = ps * r2 + ORC_S[i];
  double sr = r + (r * r2) * ps;
  double pc = ORC_C[8];
  for (int i = 7; i >= 0; i--) pc = pc * r2 + ORC_C[i];
  double cr = 1.0 + r2 * pc;
  long long q = ((long long)k) & 3;
  if (q == 0) { *sn = sr; *cs = cr; }
  else if (q == 1) { *sn = cr; *cs = -sr; }
  else if (q == 2) { *sn = -sr; *cs = -cr; }
  else { *sn = -cr; *cs = sr; }
}

/* ------------------------------------------------------------------------ */
/* Sphere-arm scenes: serial DH arms (optionally on a planar x,y,theta base) */
/* carrying collision spheres, among axis-aligned boxes.  There is no        */
/* counterpart in the reference; the primitive tests follow                  */
/* Rectangle.collides_with_sphere (abstract_env.py:69-84) and the agent-agent */
/* rule of AbstractEnvironment.is_collision_free (abstract_env.py:261-268),   */
/* applied to every pair of spheres on different robots.                      */
/* ------------------------------------------------------------------------ */
#define ORC_MAXR 16
#define ORC_MAXL 8
#define ORC_MAXJ 96

typedef struct {
  int32_t R, D, S, B;
  int32_t q_off[ORC_MAXR], base_kind[ORC_MAXR], nl[ORC_MAXR];
  double base[ORC_MAXR][12];           /* R (row-major 3x3) then p            */
  double dh[ORC_MAXR][ORC_MAXL][4];    /* a, d, cos(alpha), sin(alpha)        */
  int32_t has_off;                     /* fixed joint-angle offsets set        */
  double off[ORC_MAXJ];                /* revolute joint j turns by q[j] + off[j] */
  int32_t *s_robot, *s_link;
  double *s_loc, *s_r, *s_r2;
  double *lo, *hi;
} orc_arm;

void *orc_arm_new(int32_t R, int32_t D, const int32_t *q_off, const int32_t *base_kind,
                  const double *base_pose, const int32_t *n_links, const double *dh,
                  int32_t S, const int32_t *s_robot, const int32_t *s_link,
                  const double *s_loc, const double *s_r,
                  int32_t B, const double *box_lo, const double *box_hi) {
  if (R <= 0 || R > ORC_MAXR || S <= 0) return NULL;
  orc_arm *a = (orc_arm *)calloc(1, sizeof(orc_arm));
  a->R = R; a->D = D; a->S = S; a->B = B;
  for (int r = 0; r < R; r++) {
    if (n_links[r] > ORC_MAXL) { free(a); return NULL; }
    a->q_off[r] = q_off[r]; a->base_kind[r] = base_kind[r]; a->nl[r] = n_links[r];
    for (int i = 0; i < 12; i++) a->base[r][i] = base_pose[r * 12 + i];
    for (int l = 0; l < ORC_MAXL; l++)
      for (int i = 0; i < 4; i++) a->dh[r][l][i] = dh[(r * ORC_MAXL + l) * 4 + i];
  }
  a->s_robot = (int32_t *)malloc(sizeof(int32_t) * S);
  a->s_link = (int32_t *)malloc(sizeof(int32_t) * S);
  a->s_loc = (double *)malloc(sizeof(double) * 3 * S);
  a->s_r = (double *)malloc(sizeof(double) * S);
  a->s_r2 = (double *)malloc(sizeof(double) * S);
  memcpy(a->s_robot, s_robot, sizeof(int32_t) * S);
  memcpy(a->s_link, s_link, sizeof(int32_t) * S);
  memcpy(a->s_loc, s_loc, sizeof(double) * 3 * S);
  memcpy(a->s_r, s_r, sizeof(double) * S);
  for (int i = 0; i < S; i++) a->s_r2[i] = s_r[i] * s_r[i];
  a->lo = (double *)malloc(sizeof(double) * 3 * (B + 1));
  a->hi = (double *)malloc(sizeof(double) * 3 * (B + 1));
  if (B) { memcpy(a->lo, box_lo, sizeof(double) * 3 * B); memcpy(a->hi, box_hi, sizeof(double) * 3 * B); }
  return a;
}

/* fixed joint-angle offsets (imported general chains): joint j of the
 * configuration turns by q[j] + off[j]; NULL clears them */
int orc_arm_set_offsets(void *p, const double *off) {
  orc_arm *a = (orc_arm *)p;
  if (!a || a->D > ORC_MAXJ) return ORC_ERR_ARG;
  a->has_off = 0;
  for (int j = 0; j < a->D; j++) {
    a->off[j] = off ? off[j] : 0.0;
    if (a->off[j] != 0.0) a->has_off = 1;
  }
  return ORC_OK;
}

void orc_arm_free(void *p) {
  orc_arm *a = (orc_arm *)p;
  if (!a) return;
  free(a->s_robot); free(a->s_link); free(a->s_loc); free(a->s_r); free(a->s_r2);
  free(a->lo); free(a->hi); free(a);
}

/* World frames of robot r: frames[k] = (R 3x3, p) after k DH links; frame 0 is
 * the base (fixed pose, or planar x,y,theta followed by the mount transform). */
static void arm_frames(const orc_arm *a, int r, const double *q, double fr[ORC_MAXL + 1][12]) {
  const double *bp = a->base[r];
  int jo = a->q_off[r];
  double *R0 = fr[0];
  if (a->base_kind[r] == 1) {
    double x = q[jo], y = q[jo + 1], sn, cs;
    orc_sincos(a->has_off ? q[jo + 2] + a->off[jo + 2] : q[jo + 2], &sn, &cs);
    for (int j = 0; j < 3; j++) {
      R0[j] = cs * bp[j] - sn * bp[3 + j];
      R0[3 + j] = sn * bp[j] + cs * bp[3 + j];
      R0[6 + j] = bp[6 + j];
    }
    R0[9] = x + (cs * bp[9] - sn * bp[10]);
    R0[10] = y + (sn * bp[9] + cs * bp[10]);
    R0[11] = bp[11];
    jo += 3;
  } else {
    for (int i = 0; i < 12; i++) R0[i] = bp[i];
  }
  for (int k = 1; k <= a->nl[r]; k++) {
    const double *P = fr[k - 1];
    double *N = fr[k];
    const double *h = a->dh[r][k - 1];
    double sn, cs;
    orc_sincos(a->has_off ? q[jo + k - 1] + a->off[jo + k - 1] : q[jo + k - 1], &sn, &cs);
    double ad = h[0], dd = h[1], ca = h[2], sa = h[3];
    double sca = sn * ca, cca = cs * ca, ssa = sn * sa, csa = cs * sa;
    double ac = ad * cs, as = ad * sn;
    for (int i = 0; i < 3; i++) {
      double r0 = P[3 * i], r1 = P[3 * i + 1], r2 = P[3 * i + 2];
      N[3 * i] = r0 * cs + r1 * sn;
      N[3 * i + 1] = (r1 * cca - r0 * sca) + r2 * sa;
      N[3 * i + 2] = (r0 * ssa - r1 * csa) + r2 * ca;
      N[9 + i] = P[9 + i] + ((r0 * ac + r1 * as) + r2 * dd);
    }
  }
}

/* Sphere centres in the world frame: c = p + R * local. */
int orc_arm_fk(const void *p, const double *q, double *centers) {
  const orc_arm *a = (const orc_arm *)p;
  double fr[ORC_MAXR][ORC_MAXL + 1][12];
  for (int r = 0; r < a->R; r++) arm_frames(a, r, q, fr[r]);
  for (int s = 0; s < a->S; s++) {
    const double *F = fr[a->s_robot[s]][a->s_link[s]];
    const double *l = a->s_loc + 3 * s;
    for (int i = 0; i < 3; i++)
      centers[3 * s + i] = F[9 + i] + ((F[3 * i] * l[0] + F[3 * i + 1] * l[1]) + F[3 * i + 2] * l[2]);
  }
  return ORC_OK;
}

/* mask: bit r selects robot r (is_collision_free_for_robot: collisions of the
 * selected robots with boxes and with each other; pairs with an unselected
 * robot are ignored, rai_base_env.py:515-615); all bits: is_collision_free */
static int arm_config_free_centers_mask(const orc_arm *a, const double *c, uint32_t mask) {
  /* sphere - box: clip, squared distance summed in numpy order, <= r**2 */
  for (int s = 0; s < a->S; s++) {
    if (!((mask >> a->s_robot[s]) & 1u)) continue;
    const double *cc = c + 3 * s;
    for (int b = 0; b < a->B; b++)
      if (rect_hits(a->lo + 3 * b, a->hi + 3 * b, cc, 3, a->s_r2[s])) return 0;
  }
  /* sphere - sphere on different robots: norm(ci - cj) < ri + rj */
  for (int i = 0; i < a->S; i++)
    for (int j = i + 1; j < a->S; j++) {
      if (a->s_robot[i] == a->s_robot[j]) continue;
      if (!((mask >> a->s_robot[i]) & 1u) || !((mask >> a->s_robot[j]) & 1u)) continue;
      double d[3] = {c[3 * i] - c[3 * j], c[3 * i + 1] - c[3 * j + 1], c[3 * i + 2] - c[3 * j + 2]};
      if (sqrt(np_norm_sq(d, 3)) < a->s_r[i] + a->s_r[j]) return 0;
    }
  return 1;
}

int orc_arm_config_free_mask(const void *p, const double *q, uint32_t mask) {
  const orc_arm *a = (const orc_arm *)p;
  double *c = (double *)malloc(sizeof(double) * 3 * a->S);
  orc_arm_fk(a, q, c);
  int r = arm_config_free_centers_mask(a, c, mask);
  free(c);
  return r;
}

int orc_arm_config_free(const void *p, const double *q) { return orc_arm_config_free_mask(p, q, 0xffffffffu); }

int orc_arm_configs_free_mask(const void *scene, const double *q, int64_t n, int32_t D, uint32_t mask, uint8_t *out) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; i++) out[i] = (uint8_t)orc_arm_config_free_mask(scene, q + (size_t)i * D, mask);
  return ORC_OK;
}

/* Total penetration depth of one configuration (the library's
 * mrmg_arm_total_penetration; no reference counterpart -- the rai engine's
 * getCollisionsTotalPenetration, rai_base_env.py:464,546, on the sphere
 * model): every sphere-box overlap (radius minus the signed distance of the
 * centre to the box) and every overlap of two spheres on different robots
 * (radii minus centre distance), where positive, each rounded to a multiple
 * of 2^-40 m and summed as integers (order-independent, as on the device). */
static int64_t overlap_units(double ov) { return ov > 0.0 ? (int64_t)llrint(ov * 0x1p40) : 0; }

static double box_overlap(const double *c, const double *lo, const double *hi, double r) {
  double g2 = 0.0, dmax = -1.0e300;
  int outside = 0;
  for (int k = 0; k < 3; k++) {
    const double d = fmax(lo[k] - c[k], c[k] - hi[k]);
    dmax = fmax(dmax, d);
    if (d > 0.0) {
      g2 = g2 + d * d;
      outside = 1;
    }
  }
  return r - (outside ? sqrt(g2) : dmax);
}

int orc_arm_total_penetration(const void *scene, const double *q, int64_t n, int32_t D, double *out) {
  const orc_arm *a = (const orc_arm *)scene;
  if (!a || D != a->D) return ORC_ERR_ARG;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; i++) {
    double *c = (double *)malloc(sizeof(double) * 3 * a->S);
    orc_arm_fk(a, q + (size_t)i * D, c);
    int64_t acc = 0;
    for (int s = 0; s < a->S; s++)
      for (int b = 0; b < a->B; b++) acc += overlap_units(box_overlap(c + 3 * s, a->lo + 3 * b, a->hi + 3 * b, a->s_r[s]));
    for (int s = 0; s < a->S; s++)
      for (int t = s + 1; t < a->S; t++) {
        if (a->s_robot[s] == a->s_robot[t]) continue;
        const double dx = c[3 * s] - c[3 * t], dy = c[3 * s + 1] - c[3 * t + 1], dz = c[3 * s + 2] - c[3 * t + 2];
        acc += overlap_units((a->s_r[s] + a->s_r[t]) - sqrt((dx * dx + dy * dy) + dz * dz));
      }
    out[i] = (double)acc * 0x1p-40;
    free(c);
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Edge check  (AbstractEnvironment.is_edge_collision_free,                   */
/* problems/abstract_env.py:301-354)                                          */
/* ------------------------------------------------------------------------ */
typedef int (*config_free_fn)(const void *, const double *);

static int edge_free_impl(config_free_fn fn, const void *scene, const double *q1, const double *q2,
                          int32_t D, double res, int incl, int64_t N_in, int64_t N_start,
                          int64_t N_max, int *status, int64_t *n_checked) {
  *status = ORC_OK;
  int64_t N = N_in;
  if (N <= 0) {
    /* config_dist(q1, q2, "max") -> compute_abs_max_reduction(q1 - q2) */
    double m = fabs(q1[0] - q2[0]);
    for (int k = 1; k < D; k++) {
      double v = fabs(q1[k] - q2[k]);
      if (v > m) m = v;
    }
    double t = m / res;
    if (!(t < 9.0e15)) { *status = ORC_ERR_ARG; return 0; } /* int() of nan/inf raises */
    N = (int64_t)t + 1;
    if (N < 2) N = 2;
  }
  if (N_start > N) { *status = ORC_ERR_ARG; return 0; }
  if (N_max < 0 || N_max > N) N_max = N;
  int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)N);
  double *dir = (double *)malloc(sizeof(double) * D);
  double *q = (double *)malloc(sizeof(double) * D);
  orc_binary_indices(N, idx);
  double denom = (double)(N - 1);
  for (int k = 0; k < D; k++) dir[k] = (q2[k] - q1[k]) / denom;
  int free_ = 1;
  for (int64_t t = N_start; t < N_max; t++) {
    int64_t i = idx[t];
    if (!incl && (i == 0 || i == N - 1)) continue;
    double di = (double)i;
    for (int k = 0; k < D; k++) q[k] = q1[k] + dir[k] * di;
    if (n_checked) (*n_checked)++;
    if (!fn(scene, q)) { free_ = 0; break; }
  }
  free(idx); free(dir); free(q);
  return free_;
}

/* kind: 0 = abstract point-agent scene, 1 = sphere-arm scene */
static config_free_fn kind_fn(int kind) { return kind == 0 ? orc_abstract_config_free : orc_arm_config_free; }

int orc_edge_free(int kind, const void *scene, const double *q1, const double *q2, int32_t D,
                  double res, int incl, int64_t N_in, int64_t N_start, int64_t N_max,
                  int *status, int64_t *n_checked) {
  return edge_free_impl(kind_fn(kind), scene, q1, q2, D, res, incl, N_in, N_start, N_max, status, n_checked);
}

/* Batched forms (OpenMP over configurations / edges). */
int orc_configs_free(int kind, const void *scene, const double *q, int64_t n, int32_t D, uint8_t *out) {
  config_free_fn fn = kind_fn(kind);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; i++) out[i] = (uint8_t)fn(scene, q + (size_t)i * D);
  return ORC_OK;
}

int orc_edges_free(int kind, const void *scene, const double *q1, const double *q2, int64_t n,
                   int32_t D, double res, int incl, const int64_t *N_in, int64_t N_start,
                   int64_t N_max, uint8_t *out, int64_t *n_checked_total) {
  config_free_fn fn = kind_fn(kind);
  int bad = 0;
  int64_t tot = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : bad) reduction(+ : tot)
  for (int64_t e = 0; e < n; e++) {
    int st;
    int64_t cnt = 0;
    out[e] = (uint8_t)edge_free_impl(fn, scene, q1 + (size_t)e * D, q2 + (size_t)e * D, D, res, incl,
                                     N_in ? N_in[e] : 0, N_start, N_max, &st, &cnt);
    if (st) bad = 1;
    tot += cnt;
  }
  if (n_checked_total) *n_checked_total = tot;
  return bad ? ORC_ERR_ARG : ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Distances and costs  (problems/core/configuration.py)                     */
/* metric: 0 euclidean, 1 sum_euclidean, 2 max_euclidean, 3 max              */
/* ------------------------------------------------------------------------ */

/* compute_sliced_euclidean_dists (configuration.py:101-126), one row */
static double sliced_eucl(const double *d, int64_t s, int64_t e) {
  double acc = 0.0;
  for (int64_t k = s; k < e; k++) acc = acc + d[k] * d[k];
  return sqrt(acc);
}

/* NpConfiguration._batch_dist (configuration.py:303-329) for one row of diff */
static double dist_row(const double *d, int32_t D, const int64_t *sl, int32_t A, int metric) {
  if (metric == 0) return sliced_eucl(d, 0, sl[2 * A - 1]);
  if (metric == 1 || metric == 2) {
    double v0 = sliced_eucl(d, sl[0], sl[1]);
    if (metric == 1) {                       /* compute_sum_reduction :129-147 */
      double acc = 0.0 + v0;
      for (int i = 1; i < A; i++) acc = acc + sliced_eucl(d, sl[2 * i], sl[2 * i + 1]);
      return acc;
    }
    double m = v0;                           /* compute_max_reduction :200-219 */
    for (int i = 1; i < A; i++) {
      double v = sliced_eucl(d, sl[2 * i], sl[2 * i + 1]);
      if (v > m) m = v;
    }
    return m;
  }
  double m = fabs(d[0]);                     /* compute_abs_max_reduction :174-197 */
  for (int k = 1; k < D; k++) {
    double v = fabs(d[k]);
    if (v > m) m = v;
  }
  return m;
}

/* batch_config_dist(pt, batch, metric): out[m] = dist(pt - batch[m]) */
int orc_batch_dist(const double *pt, const double *batch, int64_t M, int32_t D, const int64_t *sl,
                   int32_t A, int metric, double *out) {
#pragma omp parallel for schedule(static) if (M > 4096)
  for (int64_t m = 0; m < M; m++) {
    double d[512];
    for (int k = 0; k < D; k++) d[k] = pt[k] - batch[(size_t)m * D + k];
    out[m] = dist_row(d, D, sl, A, metric);
  }
  return ORC_OK;
}

/* Full distance matrix: out[q, m] = batch_config_dist(queries[q], nodes)[m] */
int orc_dist_matrix(const double *qs, int64_t Q, const double *nodes, int64_t M, int32_t D,
                    const int64_t *sl, int32_t A, int metric, double *out) {
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < Q; q++) {
    double d[512];
    for (int64_t m = 0; m < M; m++) {
      for (int k = 0; k < D; k++) d[k] = qs[(size_t)q * D + k] - nodes[(size_t)m * D + k];
      out[(size_t)q * M + m] = dist_row(d, D, sl, A, metric);
    }
  }
  return ORC_OK;
}

/* _batch_config_cost_impl (configuration.py:491-510) on diff rows.
 * cost_metric: 0 euclidean, 1 max ; reduction: 0 max (max + w*sum), 1 sum */
static double cost_row(const double *d, const int64_t *sl, int32_t A, int cmetric, int red, double w) {
  double v[64];
  for (int i = 0; i < A; i++) {
    if (cmetric == 0) v[i] = sliced_eucl(d, sl[2 * i], sl[2 * i + 1]);
    else {
      double m = fabs(d[sl[2 * i]]);
      for (int64_t k = sl[2 * i] + 1; k < sl[2 * i + 1]; k++) {
        double t = fabs(d[k]);
        if (t > m || t != t) m = t;   /* np.max over |diff|: exact, NaN propagates */
      }
      v[i] = m;
    }
  }
  if (red == 0) {          /* compute_max_sum_reduction :150-171 */
    double mx = v[0], sm = v[0];
    for (int i = 1; i < A; i++) {
      if (v[i] > mx) mx = v[i];
      sm = sm + v[i];
    }
    return mx + w * sm;
  }
  double sm = 0.0;         /* compute_sum_reduction :129-147 */
  for (int i = 0; i < A; i++) sm = sm + v[i];
  return sm;
}

/* batch_config_cost (configuration.py:437-489).
 * mode 0: starts is one row broadcast against ends[M]
 * mode 1: starts[M] - ends[M]
 * mode 2: path mode, diff = starts[m+1] - starts[m], M = rows - 1      */
int orc_batch_cost(const double *starts, const double *ends, int64_t M, int32_t D, const int64_t *sl,
                   int32_t A, int cmetric, int red, double w, int mode, double *out) {
  if (A > 64 || D > 512) return ORC_ERR_ARG;
#pragma omp parallel for schedule(static) if (M > 4096)
  for (int64_t m = 0; m < M; m++) {
    double d[512];
    for (int k = 0; k < D; k++) {
      if (mode == 0) d[k] = starts[k] - ends[(size_t)m * D + k];
      else if (mode == 1) d[k] = starts[(size_t)m * D + k] - ends[(size_t)m * D + k];
      else d[k] = starts[(size_t)(m + 1) * D + k] - starts[(size_t)m * D + k];
    }
    out[m] = cost_row(d, sl, A, cmetric, red, w);
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Per-mode k nearest neighbours: the FP64 distances of batch_config_dist,   */
/* then the k smallest in (distance, index) order -- the selection of         */
/* planners/prm/prm_graph.py:446-447 (argpartition + argsort) with ties       */
/* broken by the lower index.                                                */
/* mode_off[m]..mode_off[m+1] is the node range of mode m; returned indices  */
/* are local to the query's mode.                                            */
/* ------------------------------------------------------------------------ */
int orc_knn(const double *qs, int64_t Q, const int32_t *q_mode, const double *nodes,
            const int64_t *mode_off, int32_t D, const int64_t *sl, int32_t A, int metric, int32_t k,
            int64_t *out_idx, double *out_dist) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t q = 0; q < Q; q++) {
    int64_t s = mode_off[q_mode[q]], e = mode_off[q_mode[q] + 1];
    double *bd = out_dist + (size_t)q * k;
    int64_t *bi = out_idx + (size_t)q * k;
    int cnt = 0;
    double d[512];
    for (int64_t m = s; m < e; m++) {
      for (int j = 0; j < D; j++) d[j] = qs[(size_t)q * D + j] - nodes[(size_t)m * D + j];
      double v = dist_row(d, D, sl, A, metric);
      int64_t li = m - s;
      if (cnt == k && !(v < bd[k - 1])) continue;   /* ties keep the lower index */
      int pos = cnt < k ? cnt : k - 1;
      while (pos > 0 && v < bd[pos - 1]) { bd[pos] = bd[pos - 1]; bi[pos] = bi[pos - 1]; pos--; }
      bd[pos] = v; bi[pos] = li;
      if (cnt < k) cnt++;
    }
    for (int j = cnt; j < k; j++) { bd[j] = INFINITY; bi[j] = -1; }
  }
  return ORC_OK;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
