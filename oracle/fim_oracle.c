/*
 * fim_oracle.c -- CPU FP64 restatement of the reference FIM eikonal solve path
 * (tomstrident/cufim-nvlink, src/eikonal + src/core).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU solver and
 * the timed CPU baseline of the benchmark.  The product library never links,
 * loads or calls it.
 *
 * Pinning: the local solver, the metric/edge-norm precompute and the
 * per-aggregate vertex numbering are compared bit-for-bit against the
 * reference's own code compiled on the host (oracle/_ref, built from the
 * reference sources by oracle/build.py).  The FIM state machine is pinned
 * by analytic known answers and by the reference's golden output on its unit
 * mesh (tests/golden).
 *
 * Everything is plain C11 + optional OpenMP.  Compile with
 * -ffp-contract=off so that results do not depend on whether the host
 * compiler fuses multiply-adds.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* types.h:31  "INF" of the reference is DBL_MAX, not IEEE infinity. */
#define ORC_INF DBL_MAX

/* types.h:85  enum ek_state {far, neig, narrow, next, frozen, tail, block} */
enum { ST_FAR = 0, ST_NEIG = 1, ST_NARROW = 2, ST_NEXT = 3, ST_FROZEN = 4, ST_TAIL = 5 };

/* ------------------------------------------------------------------------ */
/* Edge numbering of a tet with slots 0..3 (types.cpp:240-245):
 *   geo[0]=|x1-x0|, geo[1]=|x2-x0|, geo[2]=|x2-x1|, geo[3]=|x3-x0|,
 *   geo[4]=|x3-x1|, geo[5]=|x3-x2|  (squared M-norms).                      */
static int edge_index(int i, int j)
{
  if (i > j) { int t = i; i = j; j = t; }
  if (j == 1) return 0;
  if (j == 2) return i == 0 ? 1 : 2;
  return 3 + i; /* j == 3 */
}

/* For target slot t the reference relabels the other slots cyclically,
 * "1"=(t+1)%4, "2"=(t+2)%4, "3"=(t+3)%4, "4"=t (cuda_fim.h:41-46,
 * cuda_fim.cu:2527-2546).  sel[0..5] = geo index of the relabelled edges
 * (13, 23, 34, 12, 14, 24); oth[0..2] = slots of "1","2","3".  The tables are
 * derived here from the numbering rule instead of being written out. */
void orc_corner_tables(int t, int sel[6], int oth[3])
{
  const int s1 = (t + 1) & 3, s2 = (t + 2) & 3, s3 = (t + 3) & 3;
  sel[0] = edge_index(s1, s3); sel[1] = edge_index(s2, s3); sel[2] = edge_index(s3, t);
  sel[3] = edge_index(s1, s2); sel[4] = edge_index(s1, t);  sel[5] = edge_index(s2, t);
  oth[0] = s1; oth[1] = s2; oth[2] = s3;
}

/* ------------------------------------------------------------------------ */
/* Triangle (2-point) update, cuda_fim.h:1256-1300.  With tri_f32 != 0 the
 * intermediates are rounded to float exactly where the reference declares
 * them float; with tri_f32 == 0 everything stays in double ("pure FP64").   */
double orc_solve_tri(double e12, double e13, double e23, double p1, double p2, int tri_f32)
{
  const double a = e23;
  const double b = -0.5 * (e12 + e23 - e13);
  const double c = e12;
  const double p12 = p2 - p1;

  if (tri_f32) {
    float dv = (float)(p12 * p12 - c);
    float sv = (float)((double)dv * (b * b - a * c));
    if ((double)dv != 0.0 && (double)sv >= 0.0) {
      dv = (float)(c * (double)dv);
      const float st = sqrtf(sv);
      const float l1 = (float)(-(b * p12 * p12 - b * c - (double)st * p12) / (double)dv);
      const float l2 = (float)(-(b * p12 * p12 - b * c + (double)st * p12) / (double)dv);
      /* l1*l1 is a float product in the reference (float * float) */
      float r1 = (float)(p2 - (double)l1 * p12 + sqrt(a + 2.0 * (double)l1 * b + (double)(l1 * l1) * c));
      if (!(((double)l1 >= 0.0) && ((double)l1 <= 1.0))) r1 = (float)ORC_INF;
      float r2 = (float)(p2 - (double)l2 * p12 + sqrt(a + 2.0 * (double)l2 * b + (double)(l2 * l2) * c));
      if (!(((double)l2 >= 0.0) && ((double)l2 <= 1.0))) r2 = (float)ORC_INF;
      return (double)fminf(r1, r2);
    }
    return ORC_INF;
  } else {
    double dv = p12 * p12 - c;
    const double sv = dv * (b * b - a * c);
    if (dv != 0.0 && sv >= 0.0) {
      dv = c * dv;
      const double st = sqrt(sv);
      const double l1 = -(b * p12 * p12 - b * c - st * p12) / dv;
      const double l2 = -(b * p12 * p12 - b * c + st * p12) / dv;
      double r1 = p2 - l1 * p12 + sqrt(a + 2.0 * l1 * b + l1 * l1 * c);
      if (!((l1 >= 0.0) && (l1 <= 1.0))) r1 = HUGE_VAL;
      double r2 = p2 - l2 * p12 + sqrt(a + 2.0 * l2 * b + l2 * l2 * c);
      if (!((l2 >= 0.0) && (l2 <= 1.0))) r2 = HUGE_VAL;
      return fmin(r1, r2);
    }
    return ORC_INF;
  }
}

/* Tet (3-point) update, cuda_fim.h:1302-1360.  The reference's closed form
 * is restated term for term (it is not the exact face minimiser; the GPU
 * solver reproduces it for parity).                                         */
double orc_solve_tet(double e13, double e23, double e34, double e12, double e14, double e24,
                     double p1, double p2, double p3)
{
  const double a = e13;
  const double b = 0.5 * (e23 + e13 - e12);
  const double c = -0.5 * (e34 + e13 - e14);
  const double d = e23;
  const double e = -0.5 * (e34 + e23 - e24);
  const double f = e34;
  const double q13 = p3 - p1;
  const double q23 = p3 - p2;

  const double sqt =
    -e*e*c*d*d + a*d*d*d*d - (b*b*c - a*c*c)*f*f + ((b*b - a*c)*f*f -
    (e*e*c - a*d*d - 2.*(e*c - b*d)*e)*f)*q13*q13 - 2.*(e*e*c*d -
    2.*e*b*d*d + a*d*d*d + (b*b - a*c)*d*f)*q13*q23 + (e*e*c*c -
    2.*e*b*c*d + a*c*d*d + (b*b*c - a*c*c)*f)*q23*q23 + 2.*(e*c*d*d -
    b*d*d*d)*e + (e*e*c*c + (b*b - 2.*a*c)*d*d - 2.*(e*c*c - b*c*d)*e)*f;

  if (sqt < 0.) return ORC_INF;

  const double pa = e*c*d*d - b*d*d*d + (e*c - b*d)*f*q13*q13 - 2.*(e*c*d - b*d*d)*q13*q23 +
                    (e*c*c - b*c*d)*q23*q23 - (e*c*c - b*c*d)*f;
  const double pb = (d*d*d*d - 2.*c*d*d*f + c*c*f*f + (d*d*f - c*f*f)*q13*q13 -
                     2.*(d*d*d - c*d*f)*q13*q23 + (c*d*d - c*c*f)*q23*q23);

  const double la2 = (pa + sqt*(d*q13 - c*q23))/pb;
  const double lb2 = (pa - sqt*(d*q13 - c*q23))/pb;
  const double la1 = -((f*la2 + e)*q13 - (d*la2 + b)*q23)/(d*q13 - c*q23);
  const double lb1 = -((f*lb2 + e)*q13 - (d*lb2 + b)*q23)/(d*q13 - c*q23);

  double l3 = 1 - la1 - la2, ra = ORC_INF, rb = ORC_INF;
  if ((la1 > 0. && la1 < 1.) && (la2 > 0. && la2 < 1.) && l3 > 0.)
    ra = la1*p1 + la2*p2 + l3*p3 + sqrt(a + 2.*la1*b + la1*la1*c + 2.*la1*la2*d + 2.*la2*e + la2*la2*f);
  l3 = 1 - lb1 - lb2;
  if ((lb1 > 0. && lb1 < 1.) && (lb2 > 0. && lb2 < 1.) && l3 > 0.)
    rb = lb1*p1 + lb2*p2 + l3*p3 + sqrt(a + 2.*lb1*b + lb1*lb1*c + 2.*lb1*lb2*d + 2.*lb2*e + lb2*lb2*f);
  return fmin(ra, rb);
}

/* One corner (target slot t of a tet) update, cuda_fim.h:1362-1411.
 * ph[s] holds the time of slot s, already ORC_INF where the reference's
 * validity rule rejects the neighbour (ph[t] is ignored).                  */
double orc_corner_update(const double *geo, int t, const double *ph, int tri_f32)
{
  int sel[6], oth[3];
  orc_corner_tables(t, sel, oth);
  const double e13 = geo[sel[0]], e23 = geo[sel[1]], e34 = geo[sel[2]];
  const double e12 = geo[sel[3]], e14 = geo[sel[4]], e24 = geo[sel[5]];
  const double p1 = ph[oth[0]], p2 = ph[oth[1]], p3 = ph[oth[2]];

  double r = orc_solve_tet(e13, e23, e34, e12, e14, e24, p1, p2, p3);
  r = fmin(r, orc_solve_tri(e12, e14, e24, p1, p2, tri_f32));
  r = fmin(r, orc_solve_tri(e23, e24, e34, p2, p3, tri_f32));
  r = fmin(r, orc_solve_tri(e13, e14, e34, p1, p3, tri_f32));
  r = fmin(r, p1 + sqrt(e14));
  r = fmin(r, p2 + sqrt(e24));
  r = fmin(r, p3 + sqrt(e34));
  return r;
}

/* ------------------------------------------------------------------------ */
/* Metric precompute: compute_velocity_tensor_f3 (types.h:173-188) with the
 * per-tet speeds cf (along f) and ct (across), then the six squared M-norms of
 * compute_geo (types.cpp:227-257) in the given slot order.  load_edge(a,b)
 * is x_a - x_b (types.h:210-216).                                          */
void orc_metric_geo(int64_t nT, const int32_t *tet, const double *xyz, const double *fib,
                    const double *cf, const double *ct, double *geo)
{
  #pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nT; ++e) {
    const double *fd = fib + 3 * e;
    const double f0 = fd[0], f1 = fd[1], f2 = fd[2];
    const double fa = f0*f0, fb = f0*f1, fc = f0*f2, fdd = f1*f1, fe = f1*f2, ff = f2*f2;
    const double vf = 1. / cf[e] / cf[e], vs = 1. / ct[e] / ct[e];
    double M[6];
    M[0] = vf*fa + vs*(1. - fa);
    M[1] = (vf - vs)*fb;
    M[2] = (vf - vs)*fc;
    M[3] = vf*fdd + vs*(1. - fdd);
    M[4] = (vf - vs)*fe;
    M[5] = vf*ff + vs*(1. - ff);
    const int32_t *v = tet + 4 * e;
    static const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {1, 2, 2, 3, 3, 3};
    for (int k = 0; k < 6; ++k) {
      const double *xa = xyz + 3 * (int64_t)v[pa[k]], *xb = xyz + 3 * (int64_t)v[pb[k]];
      const double ex = xa[0] - xb[0], ey = xa[1] - xb[1], ez = xa[2] - xb[2];
      geo[6 * e + k] = (M[0]*ex + M[1]*ey + M[2]*ez)*ex +
                       (M[1]*ex + M[3]*ey + M[4]*ez)*ey +
                       (M[2]*ex + M[4]*ey + M[5]*ez)*ez;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Aggregates (submeshes) and the reference's vertex order inside a tet.
 *
 * extract_submeshes2 (types.cpp:306-570): aggregates are numbered by first
 * appearance of their tag in tet order (:331-345); local vertex ids by first
 * appearance while walking the aggregate's tets in increasing global index,
 * each tet's global ids already ascending (types.cpp:63-67 sorts them,
 * :383-398 numbers them); inside the submesh each tet's local ids are sorted
 * again (:473 -> :63-67), which fixes the slot order used by the local
 * solver.  This routine returns, per tet, its aggregate and its global vertex
 * ids in that slot order.                                                   */
typedef struct {
  int nagg;
  int32_t *agg_of_tet;     /* nT */
  int32_t *tet_slots;      /* 4*nT: global ids in reference slot order      */
  /* per aggregate CSR of local vertices (l2g) */
  int64_t *l2g_ptr;        /* nagg+1 */
  int32_t *l2g;            /* local -> global */
  int32_t *tet_local;      /* 4*nT: local ids (ascending) of each tet in its aggregate */
  int64_t *tets_ptr;       /* nagg+1, CSR of the aggregate's tets */
  int32_t *tets;           /* global tet ids in increasing order, grouped by aggregate */
} orc_aggs;

static void sort4(int32_t *a)
{
  for (int i = 1; i < 4; ++i) {
    int32_t t = a[i]; int j = i;
    for (; j > 0 && t < a[j - 1]; --j) a[j] = a[j - 1];
    a[j] = t;
  }
}

static int orc_build_aggs(int nV, int64_t nT, const int32_t *tets_in, const int32_t *atags, orc_aggs *A)
{
  memset(A, 0, sizeof(*A));
  A->agg_of_tet = malloc(sizeof(int32_t) * nT);
  A->tet_slots = malloc(sizeof(int32_t) * 4 * nT);
  A->tet_local = malloc(sizeof(int32_t) * 4 * nT);
  A->tets = malloc(sizeof(int32_t) * nT);
  if (!A->agg_of_tet || !A->tet_slots || !A->tet_local || !A->tets) return -1;

  /* tag -> aggregate index by first appearance (std::map lookup order is
   * irrelevant; the numbering is first appearance). Tags may be arbitrary
   * ints: use a sorted table of (tag, agg). */
  int cap = 16, n = 0;
  int32_t *tagv = malloc(sizeof(int32_t) * cap), *aggv = malloc(sizeof(int32_t) * cap);
  for (int64_t e = 0; e < nT; ++e) {
    const int32_t tg = atags ? atags[e] : 0;
    int lo = 0, hi = n;
    while (lo < hi) { int mid = (lo + hi) / 2; if (tagv[mid] < tg) lo = mid + 1; else hi = mid; }
    if (lo < n && tagv[lo] == tg) { A->agg_of_tet[e] = aggv[lo]; continue; }
    if (n == cap) { cap *= 2; tagv = realloc(tagv, sizeof(int32_t) * cap); aggv = realloc(aggv, sizeof(int32_t) * cap); }
    memmove(tagv + lo + 1, tagv + lo, sizeof(int32_t) * (n - lo));
    memmove(aggv + lo + 1, aggv + lo, sizeof(int32_t) * (n - lo));
    tagv[lo] = tg; aggv[lo] = A->nagg; A->agg_of_tet[e] = A->nagg; A->nagg++; n++;
  }
  free(tagv); free(aggv);
  const int na = A->nagg;

  A->tets_ptr = calloc(na + 1, sizeof(int64_t));
  for (int64_t e = 0; e < nT; ++e) A->tets_ptr[A->agg_of_tet[e] + 1]++;
  for (int a = 0; a < na; ++a) A->tets_ptr[a + 1] += A->tets_ptr[a];
  int64_t *fill = malloc(sizeof(int64_t) * na);
  for (int a = 0; a < na; ++a) fill[a] = A->tets_ptr[a];
  for (int64_t e = 0; e < nT; ++e) A->tets[fill[A->agg_of_tet[e]]++] = (int32_t)e;

  /* local numbering per aggregate */
  int32_t *g2l = malloc(sizeof(int32_t) * nV);
  for (int i = 0; i < nV; ++i) g2l[i] = -1;
  A->l2g_ptr = calloc(na + 1, sizeof(int64_t));
  int64_t l2g_cap = nV + 16, l2g_n = 0;
  A->l2g = malloc(sizeof(int32_t) * l2g_cap);
  for (int a = 0; a < na; ++a) {
    int32_t nl = 0;
    const int64_t base = l2g_n;
    for (int64_t k = A->tets_ptr[a]; k < A->tets_ptr[a + 1]; ++k) {
      const int64_t e = A->tets[k];
      int32_t g[4];
      memcpy(g, tets_in + 4 * e, sizeof(g));
      sort4(g);
      int32_t l[4];
      for (int s = 0; s < 4; ++s) {
        if (g2l[g[s]] < 0) {
          if (l2g_n == l2g_cap) { l2g_cap *= 2; A->l2g = realloc(A->l2g, sizeof(int32_t) * l2g_cap); }
          g2l[g[s]] = nl++;
          A->l2g[l2g_n++] = g[s];
        }
        l[s] = g2l[g[s]];
      }
      sort4(l);
      for (int s = 0; s < 4; ++s) {
        A->tet_local[4 * e + s] = l[s];
        A->tet_slots[4 * e + s] = A->l2g[base + l[s]];
      }
    }
    A->l2g_ptr[a + 1] = l2g_n;
    for (int64_t i = base; i < l2g_n; ++i) g2l[A->l2g[i]] = -1;
  }
  free(g2l); free(fill);
  return 0;
}

static void orc_free_aggs(orc_aggs *A)
{
  free(A->agg_of_tet); free(A->tet_slots); free(A->tet_local);
  free(A->tets_ptr); free(A->tets); free(A->l2g_ptr); free(A->l2g);
  memset(A, 0, sizeof(*A));
}

/* Public: slot order of every tet (and its aggregate) for a partition. */
int orc_reference_slots(int nV, int64_t nT, const int32_t *tets, const int32_t *atags,
                        int32_t *tet_slots, int32_t *agg_of_tet, int32_t *tet_local)
{
  orc_aggs A;
  if (orc_build_aggs(nV, nT, tets, atags, &A)) return -1;
  memcpy(tet_slots, A.tet_slots, sizeof(int32_t) * 4 * nT);
  if (agg_of_tet) memcpy(agg_of_tet, A.agg_of_tet, sizeof(int32_t) * nT);
  if (tet_local) memcpy(tet_local, A.tet_local, sizeof(int32_t) * 4 * nT);
  const int na = A.nagg;
  orc_free_aggs(&A);
  return na;
}

/* ------------------------------------------------------------------------ */
/* Submesh connectivity (compute_base_connectivity, types.cpp:43-225) in
 * local ids: n2e in increasing local-tet order, n2n = sorted union of the
 * vertices of the incident tets (self included).                            */
typedef struct {
  int32_t nn, ne;
  const int32_t *gid;       /* local -> global vertex */
  int32_t *tv;              /* 4*ne local ids, ascending */
  const double *geo;        /* 6*ne, slot order */
  int64_t *n2e_ptr; int32_t *n2e;   /* tet index per (vertex, entry)  */
  int64_t *n2n_ptr; int32_t *n2n;
  /* state */
  double *phi; int32_t *st; int32_t *tst; double *tphi;
} orc_sub;

static int cmp_i32(const void *a, const void *b)
{
  const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

static void orc_sub_connect(orc_sub *S)
{
  S->n2e_ptr = calloc(S->nn + 1, sizeof(int64_t));
  for (int32_t e = 0; e < S->ne; ++e)
    for (int s = 0; s < 4; ++s) S->n2e_ptr[S->tv[4 * e + s] + 1]++;
  for (int32_t v = 0; v < S->nn; ++v) S->n2e_ptr[v + 1] += S->n2e_ptr[v];
  S->n2e = malloc(sizeof(int32_t) * (S->n2e_ptr[S->nn] + 1));
  int64_t *fill = malloc(sizeof(int64_t) * (S->nn + 1));
  for (int32_t v = 0; v < S->nn; ++v) fill[v] = S->n2e_ptr[v];
  for (int32_t e = 0; e < S->ne; ++e)
    for (int s = 0; s < 4; ++s) { const int32_t v = S->tv[4 * e + s]; S->n2e[fill[v]++] = e; }
  /* n2n: union of tet vertices, sorted unique */
  S->n2n_ptr = calloc(S->nn + 1, sizeof(int64_t));
  /* gather buffer: four ids per incident tet of the busiest vertex */
  int64_t maxdeg = 0;
  for (int32_t v = 0; v < S->nn; ++v)
    if (S->n2e_ptr[v + 1] - S->n2e_ptr[v] > maxdeg) maxdeg = S->n2e_ptr[v + 1] - S->n2e_ptr[v];
  int32_t *buf = malloc(sizeof(int32_t) * (size_t)(4 * maxdeg + 1));
  int64_t cap = (int64_t)S->nn * 16 + 16, used = 0;
  S->n2n = malloc(sizeof(int32_t) * cap);
  for (int32_t v = 0; v < S->nn; ++v) {
    int nb = 0;
    for (int64_t k = S->n2e_ptr[v]; k < S->n2e_ptr[v + 1]; ++k)
      for (int s = 0; s < 4; ++s) buf[nb++] = S->tv[4 * S->n2e[k] + s];
    qsort(buf, nb, sizeof(int32_t), cmp_i32);
    int m = 0;
    for (int i = 0; i < nb; ++i) if (m == 0 || buf[i] != buf[m - 1]) buf[m++] = buf[i];
    if (used + m > cap) { cap = 2 * (used + m); S->n2n = realloc(S->n2n, sizeof(int32_t) * cap); }
    memcpy(S->n2n + used, buf, sizeof(int32_t) * m);
    used += m;
    S->n2n_ptr[v + 1] = used;
  }
  free(buf); free(fill);
}

static void orc_sub_free(orc_sub *S)
{
  free(S->tv); free(S->n2e_ptr); free(S->n2e); free(S->n2n_ptr); free(S->n2n);
  free(S->phi); free(S->st); free(S->tst); free(S->tphi);
  free((void *)S->geo);
}

/* update_per_element (cuda_fim.h:1362-1411) on a submesh. */
static double sub_update(const orc_sub *S, int32_t v, int32_t e, double phi_start, double fw, int tri_f32)
{
  double ph[4];
  int t = 0;
  for (int s = 0; s < 4; ++s) {
    const int32_t n = S->tv[4 * e + s];
    if (n == v) { t = s; ph[s] = 0.0; }
    else if (S->st[n] >= ST_NARROW && S->phi[n] > (phi_start - fw)) ph[s] = S->phi[n];
    else ph[s] = ORC_INF;
  }
  return orc_corner_update(S->geo + 6 * (int64_t)e, t, ph, tri_f32);
}

/* update_states (cuda_fim.cu:1790-1845); apd_us is the hard-coded 3e5. */
static int sub_update_states(orc_sub *S, double cur_time, double apd_us)
{
  int active = 0;
  for (int32_t v = 0; v < S->nn; ++v) {
    const int st = S->st[v];
    if (st == ST_NARROW) active++;
    else if (st == ST_NEXT) { active++; S->st[v] = ST_NARROW; }
    else if (st == ST_FROZEN) { if (!(S->phi[v] + apd_us > cur_time)) S->st[v] = ST_TAIL; }
    else if (st == ST_TAIL) {
      if (!(S->phi[v] + apd_us / 0.91 > cur_time)) { S->phi[v] = ORC_INF; S->st[v] = ST_FAR; }
    }
  }
  return active;
}

/* compute_step (cuda_fim.cu:1992-2334) for one submesh, phases executed
 * with block-synchronous (snapshot) semantics.  The reference reads
 * tmp_state of neighbours in the marking phase while other threads write it
 * (:2196 vs :2200); here the marking phase reads the values from before the
 * phase, which is what the phase would see without that race.               */
static long sub_compute_step(orc_sub *S, double fw, double cur_time, double phi_start, double dt,
                             double apd_us, int tri_f32, int max_iter)
{
  int active = sub_update_states(S, cur_time, apd_us);
  long iters = 0;
  int32_t *tst_snap = malloc(sizeof(int32_t) * (S->nn + 1));
  while (active > 0) {
    if (max_iter > 0 && iters >= max_iter) break;
    iters++;
    active = 0;
    /* solve on elements */
    for (int32_t v = 0; v < S->nn; ++v)
      for (int64_t k = S->n2e_ptr[v]; k < S->n2e_ptr[v + 1]; ++k)
        S->tphi[k] = (S->st[v] == ST_NARROW) ? sub_update(S, v, S->n2e[k], phi_start, fw, tri_f32) : ORC_INF;
    /* reduce per vertex */
    for (int32_t v = 0; v < S->nn; ++v) {
      S->tst[v] = ST_FAR;
      if (S->st[v] != ST_NARROW) continue;
      const double old = S->phi[v];
      double nw = old;
      for (int64_t k = S->n2e_ptr[v]; k < S->n2e_ptr[v + 1]; ++k) if (S->tphi[k] < nw) nw = S->tphi[k];
      S->phi[v] = nw;
      if (nw - phi_start > dt) S->st[v] = ST_NEXT;
      else if (fabs(old - nw) < (1e-6 * (1 + (old + nw) * .5))) S->tst[v] = ST_FROZEN;
    }
    /* mark neighbours */
    memcpy(tst_snap, S->tst, sizeof(int32_t) * S->nn);
    for (int32_t v = 0; v < S->nn; ++v) {
      if (S->st[v] == ST_NARROW) continue;
      for (int64_t k = S->n2n_ptr[v]; k < S->n2n_ptr[v + 1]; ++k) {
        const int32_t n = S->n2n[k];
        if (tst_snap[n] == ST_FROZEN && S->phi[n] < S->phi[v]) {
          S->tst[v] = S->st[v];
          S->st[v] = ST_NEIG;
          break;
        }
      }
    }
    /* solve elements for neighbours */
    for (int32_t v = 0; v < S->nn; ++v)
      for (int64_t k = S->n2e_ptr[v]; k < S->n2e_ptr[v + 1]; ++k)
        S->tphi[k] = (S->st[v] == ST_NEIG) ? sub_update(S, v, S->n2e[k], phi_start, fw, tri_f32) : ORC_INF;
    /* reduce neighbours */
    for (int32_t v = 0; v < S->nn; ++v) {
      if (S->st[v] != ST_NEIG) continue;
      const double old = S->phi[v];
      double nw = old;
      for (int64_t k = S->n2e_ptr[v]; k < S->n2e_ptr[v + 1]; ++k) if (S->tphi[k] < nw) nw = S->tphi[k];
      S->phi[v] = nw;
      S->st[v] = (nw < old) ? ST_NARROW : S->tst[v];
    }
    /* update neighbour states */
    for (int32_t v = 0; v < S->nn; ++v) {
      if (S->st[v] == ST_NARROW) {
        if (S->tst[v] == ST_FROZEN) S->st[v] = ST_FROZEN; else active++;
      } else if (S->st[v] == ST_NEIG) { S->st[v] = ST_NARROW; active++; }
    }
  }
  free(tst_snap);
  return iters;
}

/* ------------------------------------------------------------------------ */
/* Reference-semantics solve (CudaSolverFIM::solve, cuda_fim.cu:2386-2503):
 *   reset (reset_states_gpu :479-542), seed (update_events_gpu :632-683; the
 *   reference seeds phi = 0 -- the caller passes t0 = 0 for that),
 *   then n_steps x { sync_step2 (:1752-1787); compute_step }, then the
 *   local -> global gather (min phi, max state, :2466-2485).
 * tets are global ids (any order); atags NULL = one aggregate.
 * geo_slots is 6*nT in the reference slot order (orc_reference_slots).     */
long orc_solve_reference(int nV, int64_t nT, const int32_t *tets, const int32_t *atags,
                         const double *geo_slots, int nseed, const int32_t *seed_v, const double *seed_t,
                         double dt, int n_steps, double fw, double apd_us, int tri_f32, int max_iter,
                         double *phi_out, int32_t *state_out)
{
  orc_aggs A;
  if (orc_build_aggs(nV, nT, tets, atags, &A)) return -1;
  const int na = A.nagg;
  orc_sub *S = calloc(na, sizeof(orc_sub));
  for (int a = 0; a < na; ++a) {
    orc_sub *s = &S[a];
    s->nn = (int32_t)(A.l2g_ptr[a + 1] - A.l2g_ptr[a]);
    s->ne = (int32_t)(A.tets_ptr[a + 1] - A.tets_ptr[a]);
    s->gid = A.l2g + A.l2g_ptr[a];
    s->tv = malloc(sizeof(int32_t) * 4 * (s->ne + 1));
    double *g = malloc(sizeof(double) * 6 * (s->ne + 1));
    for (int32_t k = 0; k < s->ne; ++k) {
      const int64_t e = A.tets[A.tets_ptr[a] + k];
      memcpy(s->tv + 4 * k, A.tet_local + 4 * e, sizeof(int32_t) * 4);
      memcpy(g + 6 * k, geo_slots + 6 * e, sizeof(double) * 6);
    }
    s->geo = g;
    orc_sub_connect(s);
    s->phi = malloc(sizeof(double) * (s->nn + 1));
    s->st = malloc(sizeof(int32_t) * (s->nn + 1));
    s->tst = malloc(sizeof(int32_t) * (s->nn + 1));
    s->tphi = malloc(sizeof(double) * (s->n2e_ptr[s->nn] + 1));
    for (int32_t v = 0; v < s->nn; ++v) { s->phi[v] = ORC_INF; s->st[v] = ST_FAR; s->tst[v] = ST_FAR; }
  }
  /* global vertex -> list of (agg, local) copies, in aggregate order */
  int64_t *cp_ptr = calloc(nV + 1, sizeof(int64_t));
  for (int a = 0; a < na; ++a)
    for (int32_t l = 0; l < S[a].nn; ++l) cp_ptr[S[a].gid[l] + 1]++;
  for (int v = 0; v < nV; ++v) cp_ptr[v + 1] += cp_ptr[v];
  int32_t *cp_a = malloc(sizeof(int32_t) * (cp_ptr[nV] + 1)), *cp_l = malloc(sizeof(int32_t) * (cp_ptr[nV] + 1));
  int64_t *fill = malloc(sizeof(int64_t) * (nV + 1));
  for (int v = 0; v < nV; ++v) fill[v] = cp_ptr[v];
  for (int a = 0; a < na; ++a)
    for (int32_t l = 0; l < S[a].nn; ++l) { const int32_t g = S[a].gid[l]; cp_a[fill[g]] = a; cp_l[fill[g]] = l; fill[g]++; }

  /* seeds: every copy of the vertex */
  for (int i = 0; i < nseed; ++i) {
    const int32_t g = seed_v[i];
    if (g < 0 || g >= nV) continue;
    for (int64_t k = cp_ptr[g]; k < cp_ptr[g + 1]; ++k) {
      orc_sub *s = &S[cp_a[k]];
      s->phi[cp_l[k]] = seed_t[i];
      s->st[cp_l[k]] = ST_NARROW;
    }
  }

  long iters = 0;
  double cur_time = 0.0, phi_start = 0.0;
  for (int step = 0; step < n_steps; ++step) {
    phi_start = cur_time;
    cur_time += dt;
    /* sync_step2 */
    for (int v = 0; v < nV; ++v) {
      double nw = ORC_INF;
      for (int64_t k = cp_ptr[v]; k < cp_ptr[v + 1]; ++k) { const double p = S[cp_a[k]].phi[cp_l[k]]; if (p < nw) nw = p; }
      for (int64_t k = cp_ptr[v]; k < cp_ptr[v + 1]; ++k) {
        orc_sub *s = &S[cp_a[k]];
        if (nw < s->phi[cp_l[k]]) { s->phi[cp_l[k]] = nw; s->st[cp_l[k]] = ST_NARROW; }
      }
    }
    for (int a = 0; a < na; ++a)
      iters += sub_compute_step(&S[a], fw, cur_time, phi_start, dt, apd_us, tri_f32, max_iter);
  }
  /* gather */
  for (int v = 0; v < nV; ++v) { phi_out[v] = ORC_INF; if (state_out) state_out[v] = ST_FAR; }
  for (int a = 0; a < na; ++a)
    for (int32_t l = 0; l < S[a].nn; ++l) {
      const int32_t g = S[a].gid[l];
      if (S[a].phi[l] < phi_out[g]) phi_out[g] = S[a].phi[l];
      if (state_out && S[a].st[l] > state_out[g]) state_out[g] = S[a].st[l];
    }
  for (int a = 0; a < na; ++a) orc_sub_free(&S[a]);
  free(S); free(cp_ptr); free(cp_a); free(cp_l); free(fill);
  orc_free_aggs(&A);
  return iters;
}

/* ------------------------------------------------------------------------ */
/* Single-aggregate, single-window FIM with active lists (the "pure" mode:
 * one submesh, dt = +inf, one step).  Same phases and the same arithmetic as
 * sub_compute_step, but each phase touches only the narrow list, the newly
 * frozen vertices and their neighbours, so it scales to million-vertex
 * meshes; OpenMP parallelises the local solves.  Used as the timed CPU
 * baseline and as the FP64 oracle of the large configurations.
 * tet_slots: 4*nT global ids in slot order; geo 6*nT in that order.        */
typedef struct {
  int nV; int64_t nT;
  const int32_t *tv; const double *geo;
  int64_t *n2e_ptr; int32_t *n2e;
  int64_t *n2n_ptr; int32_t *n2n;
} orc_mesh;

static int orc_mesh_build(orc_mesh *M, int nV, int64_t nT, const int32_t *tv, const double *geo)
{
  memset(M, 0, sizeof(*M));
  M->nV = nV; M->nT = nT; M->tv = tv; M->geo = geo;
  M->n2e_ptr = calloc((size_t)nV + 1, sizeof(int64_t));
  for (int64_t e = 0; e < nT; ++e) for (int s = 0; s < 4; ++s) M->n2e_ptr[tv[4 * e + s] + 1]++;
  for (int v = 0; v < nV; ++v) M->n2e_ptr[v + 1] += M->n2e_ptr[v];
  M->n2e = malloc(sizeof(int32_t) * (M->n2e_ptr[nV] + 1));
  int64_t *fill = malloc(sizeof(int64_t) * ((size_t)nV + 1));
  for (int v = 0; v < nV; ++v) fill[v] = M->n2e_ptr[v];
  for (int64_t e = 0; e < nT; ++e) for (int s = 0; s < 4; ++s) { const int32_t v = tv[4 * e + s]; M->n2e[fill[v]++] = (int32_t)e; }
  free(fill);
  M->n2n_ptr = calloc((size_t)nV + 1, sizeof(int64_t));
  int32_t *cnt = calloc((size_t)nV + 1, sizeof(int32_t));
  /* gather buffer: four ids per incident tet of the busiest vertex */
  int64_t maxdeg = 0;
  for (int v = 0; v < nV; ++v)
    if (M->n2e_ptr[v + 1] - M->n2e_ptr[v] > maxdeg) maxdeg = M->n2e_ptr[v + 1] - M->n2e_ptr[v];
  const size_t bufn = (size_t)(4 * maxdeg + 1);
  /* two passes: count unique, then fill */
  #pragma omp parallel
  {
    int32_t *buf = malloc(sizeof(int32_t) * bufn);
    #pragma omp for schedule(static)
    for (int v = 0; v < nV; ++v) {
      int nb = 0;
      for (int64_t k = M->n2e_ptr[v]; k < M->n2e_ptr[v + 1]; ++k)
        for (int s = 0; s < 4; ++s) buf[nb++] = tv[4 * (int64_t)M->n2e[k] + s];
      qsort(buf, nb, sizeof(int32_t), cmp_i32);
      int m = 0;
      for (int i = 0; i < nb; ++i) if (m == 0 || buf[i] != buf[m - 1]) buf[m++] = buf[i];
      cnt[v] = m;
    }
    free(buf);
  }
  for (int v = 0; v < nV; ++v) M->n2n_ptr[v + 1] = M->n2n_ptr[v] + cnt[v];
  M->n2n = malloc(sizeof(int32_t) * (M->n2n_ptr[nV] + 1));
  #pragma omp parallel
  {
    int32_t *buf = malloc(sizeof(int32_t) * bufn);
    #pragma omp for schedule(static)
    for (int v = 0; v < nV; ++v) {
      int nb = 0;
      for (int64_t k = M->n2e_ptr[v]; k < M->n2e_ptr[v + 1]; ++k)
        for (int s = 0; s < 4; ++s) buf[nb++] = tv[4 * (int64_t)M->n2e[k] + s];
      qsort(buf, nb, sizeof(int32_t), cmp_i32);
      int m = 0;
      for (int i = 0; i < nb; ++i) if (m == 0 || buf[i] != buf[m - 1]) buf[m++] = buf[i];
      memcpy(M->n2n + M->n2n_ptr[v], buf, sizeof(int32_t) * m);
    }
    free(buf);
  }
  free(cnt);
  return 0;
}

static void orc_mesh_free(orc_mesh *M)
{
  free(M->n2e_ptr); free(M->n2e); free(M->n2n_ptr); free(M->n2n);
}

static double mesh_vertex_update(const orc_mesh *M, const double *phi, const int32_t *st, int32_t v,
                                 double phi_start, double fw, int tri_f32)
{
  double nw = phi[v];
  for (int64_t k = M->n2e_ptr[v]; k < M->n2e_ptr[v + 1]; ++k) {
    const int32_t e = M->n2e[k];
    double ph[4]; int t = 0;
    for (int s = 0; s < 4; ++s) {
      const int32_t n = M->tv[4 * (int64_t)e + s];
      if (n == v) { t = s; ph[s] = 0.0; }
      else if (st[n] >= ST_NARROW && phi[n] > (phi_start - fw)) ph[s] = phi[n];
      else ph[s] = ORC_INF;
    }
    const double c = orc_corner_update(M->geo + 6 * (int64_t)e, t, ph, tri_f32);
    if (c < nw) nw = c;
  }
  return nw;
}

/* Local support of a finished solve: U[v] = the minimum over every corner
 * of v of the reference's local update (update_per_element,
 * cuda_fim.h:1362-1411) from the final times and states of its neighbours,
 * not counting v's own time (INF where no corner gives a value).  A time
 * below its U is not attained by any candidate from its neighbours. */
void orc_support(int nV, int64_t nT, const int32_t *tet_slots, const double *geo_slots, const double *phi,
                 const int32_t *state, int tri_f32, double *U)
{
  orc_mesh M;
  orc_mesh_build(&M, nV, nT, tet_slots, geo_slots);
  #pragma omp parallel for schedule(dynamic, 256)
  for (int v = 0; v < nV; ++v) {
    double nw = ORC_INF;
    for (int64_t k = M.n2e_ptr[v]; k < M.n2e_ptr[v + 1]; ++k) {
      const int32_t e = M.n2e[k];
      double ph[4]; int t = 0;
      for (int s = 0; s < 4; ++s) {
        const int32_t n = M.tv[4 * (int64_t)e + s];
        if (n == v) { t = s; ph[s] = 0.0; }
        else if (state[n] >= ST_NARROW) ph[s] = phi[n];
        else ph[s] = ORC_INF;
      }
      const double c = orc_corner_update(M.geo + 6 * (int64_t)e, t, ph, tri_f32);
      if (c < nw) nw = c;
    }
    U[v] = nw;
  }
  orc_mesh_free(&M);
}

long orc_solve_pure(int nV, int64_t nT, const int32_t *tet_slots, const double *geo_slots,
                    int nseed, const int32_t *seed_v, const double *seed_t, int tri_f32,
                    int threads, long max_iter, double *phi, int32_t *state_out, long *n_updates)
{
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  orc_mesh M;
  orc_mesh_build(&M, nV, nT, tet_slots, geo_slots);
  const double phi_start = 0.0, fw = HUGE_VAL, dt = HUGE_VAL;
  int32_t *st = malloc(sizeof(int32_t) * nV), *tst = malloc(sizeof(int32_t) * nV);
  int32_t *narrow = malloc(sizeof(int32_t) * nV), *marked = malloc(sizeof(int32_t) * nV);
  int32_t *frozen_now = malloc(sizeof(int32_t) * nV);
  uint8_t *flag = calloc(nV, 1);
  double *nwv = malloc(sizeof(double) * nV);
  for (int v = 0; v < nV; ++v) { phi[v] = ORC_INF; st[v] = ST_FAR; tst[v] = ST_FAR; }
  int nn = 0;
  for (int i = 0; i < nseed; ++i) {
    const int32_t g = seed_v[i];
    if (g < 0 || g >= nV) continue;
    phi[g] = seed_t[i];
    if (st[g] != ST_NARROW) { st[g] = ST_NARROW; narrow[nn++] = g; }
  }
  long iters = 0, upd = 0;
  /* One window that never closes: dt = inf, so no vertex becomes "next",
   * and the front-width rule phi > phi_start - fw passes for every finite
   * time (fw = inf).  There is one step, so update_states only promotes the
   * seeds, which are narrow already. */
  while (nn > 0) {
    if (max_iter > 0 && iters >= max_iter) break;
    iters++;
    upd += nn;
    /* (a)+(b): candidates for the narrow list from the snapshot */
    #pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < nn; ++i) nwv[i] = mesh_vertex_update(&M, phi, st, narrow[i], phi_start, fw, tri_f32);
    int nf = 0;
    for (int i = 0; i < nn; ++i) {
      const int32_t v = narrow[i];
      const double old = phi[v], nw = nwv[i];
      tst[v] = ST_FAR;
      phi[v] = nw;
      if (nw - phi_start > dt) st[v] = ST_NEXT;
      else if (fabs(old - nw) < (1e-6 * (1 + (old + nw) * .5))) { tst[v] = ST_FROZEN; frozen_now[nf++] = v; }
    }
    /* (c): non-narrow neighbours of newly frozen vertices with larger phi */
    int nm = 0;
    for (int i = 0; i < nf; ++i) {
      const int32_t n = frozen_now[i];
      for (int64_t k = M.n2n_ptr[n]; k < M.n2n_ptr[n + 1]; ++k) {
        const int32_t v = M.n2n[k];
        if (st[v] == ST_NARROW || flag[v]) continue;
        if (phi[n] < phi[v]) { flag[v] = 1; marked[nm++] = v; }
      }
    }
    for (int i = 0; i < nm; ++i) { const int32_t v = marked[i]; tst[v] = st[v]; st[v] = ST_NEIG; }
    /* (d)+(e) */
    upd += nm;
    #pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < nm; ++i) nwv[i] = mesh_vertex_update(&M, phi, st, marked[i], phi_start, fw, tri_f32);
    for (int i = 0; i < nm; ++i) {
      const int32_t v = marked[i];
      const double old = phi[v], nw = nwv[i];
      phi[v] = nw;
      st[v] = (nw < old) ? ST_NARROW : tst[v];
      flag[v] = 0;
    }
    /* (f): new narrow list.  Vertices of the old list first, then marked
     * ones that did not come from the old list. */
    int nn2 = 0;
    for (int i = 0; i < nn; ++i) {
      const int32_t v = narrow[i];
      if (st[v] == ST_NARROW) {
        if (tst[v] == ST_FROZEN) st[v] = ST_FROZEN;
        else if (!flag[v]) { flag[v] = 1; frozen_now[nn2++] = v; }
      }
    }
    for (int i = 0; i < nm; ++i) {
      const int32_t v = marked[i];
      if (st[v] == ST_NARROW) {
        if (tst[v] == ST_FROZEN) st[v] = ST_FROZEN;
        else if (!flag[v]) { flag[v] = 1; frozen_now[nn2++] = v; }
      }
    }
    for (int i = 0; i < nn2; ++i) { narrow[i] = frozen_now[i]; flag[narrow[i]] = 0; }
    nn = nn2;
  }
  if (state_out) memcpy(state_out, st, sizeof(int32_t) * nV);
  if (n_updates) *n_updates = upd;
  free(st); free(tst); free(narrow); free(marked); free(frozen_now); free(flag); free(nwv);
  orc_mesh_free(&M);
  return iters;
}

/* ------------------------------------------------------------------------ */
/* Exact fixed point of the same local update (analysis tool): label
 * correcting with Jacobi sweeps over the vertices whose neighbourhood
 * changed, every neighbour with a finite time counted valid, until no time
 * decreases.  Starts from phi_init (e.g. the FIM result) if given.          */
long orc_fixed_point(int nV, int64_t nT, const int32_t *tet_slots, const double *geo_slots,
                     int nseed, const int32_t *seed_v, const double *seed_t, int tri_f32,
                     int threads, long max_sweeps, const double *phi_init, double *phi)
{
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  orc_mesh M;
  orc_mesh_build(&M, nV, nT, tet_slots, geo_slots);
  int32_t *st = malloc(sizeof(int32_t) * nV);
  uint8_t *act = calloc(nV, 1), *nxt = calloc(nV, 1);
  double *nw = malloc(sizeof(double) * nV);
  for (int v = 0; v < nV; ++v) { phi[v] = phi_init ? phi_init[v] : ORC_INF; }
  for (int i = 0; i < nseed; ++i) if (seed_v[i] >= 0 && seed_v[i] < nV && seed_t[i] < phi[seed_v[i]]) phi[seed_v[i]] = seed_t[i];
  for (int v = 0; v < nV; ++v) { st[v] = phi[v] < ORC_INF ? ST_FROZEN : ST_FAR; act[v] = 1; }
  long sweeps = 0;
  for (;;) {
    if (max_sweeps > 0 && sweeps >= max_sweeps) break;
    sweeps++;
    long changed = 0;
    #pragma omp parallel for schedule(dynamic, 256) reduction(+:changed)
    for (int v = 0; v < nV; ++v) {
      nw[v] = phi[v];
      if (!act[v]) continue;
      const double c = mesh_vertex_update(&M, phi, st, v, 0.0, HUGE_VAL, tri_f32);
      if (c < phi[v]) { nw[v] = c; changed++; }
    }
    if (!changed) break;
    memset(nxt, 0, nV);
    for (int v = 0; v < nV; ++v) {
      if (nw[v] < phi[v]) {
        for (int64_t k = M.n2n_ptr[v]; k < M.n2n_ptr[v + 1]; ++k) nxt[M.n2n[k]] = 1;
      }
    }
    for (int v = 0; v < nV; ++v) { if (nw[v] < phi[v]) { phi[v] = nw[v]; st[v] = ST_FROZEN; } }
    uint8_t *t = act; act = nxt; nxt = t;
  }
  free(st); free(act); free(nxt); free(nw);
  orc_mesh_free(&M);
  return sweeps;
}

/* Reference front width (compute_dwf, cuda_fim.h:1536-1576):
 * 1.01 * longest Euclidean edge / 0.6.  Edges are enumerated per tet, which
 * covers every n2n pair.                                                    */
double orc_front_width(int64_t nT, const int32_t *tets, const double *xyz, double speed)
{
  double m = 0.0;
  for (int64_t e = 0; e < nT; ++e)
    for (int i = 0; i < 4; ++i)
      for (int j = i + 1; j < 4; ++j) {
        const double *a = xyz + 3 * (int64_t)tets[4 * e + i], *b = xyz + 3 * (int64_t)tets[4 * e + j];
        const double dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
        const double l = dx * dx + dy * dy + dz * dz;
        if (l > m) m = l;
      }
  return 1.01 * sqrt(m) / speed;
}
