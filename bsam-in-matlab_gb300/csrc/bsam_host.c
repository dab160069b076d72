/*
 * bsam_host.c -- host-side helpers for hierarchy set-up (not the solve path).
 *
 *  - Vectorised C-library math (exp, tanh, cosh, sin, cos, atan2, hypot,
 *    sqrt) so coefficient sampling gives the same bits on every host,
 *    independent of a vector-math library's approximations.
 *  - The starfish polygon geometry of DiffuseDomainBSAM/src/ddStarfishGeometry.m:
 *    the radially sampled closed polygon, a bounding-box tree over its
 *    segments (midpoint splits; leaves of at most 16 segments where the
 *    reference's have 8 -- the tree's shape decides only how much is
 *    pruned, never the minimum), and the exact point-to-segment signed
 *    distance with the reference's pruning rule (prune when the box
 *    distance exceeds the current best plus 64 eps).  The sign comes from
 *    the radial-ray intersection with the enclosing segment.
 *
 * Compiled with -ffp-contract=off -fno-fast-math (at -O3) so the arithmetic
 * is the same on x86-64 and aarch64 hosts: no contraction, no reassociation,
 * no vector math library.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

#define VEC1(name, fn) \
  void bsam_v##name(const double *x, double *y, int64_t n) { for (int64_t i = 0; i < n; ++i) y[i] = fn(x[i]); }
VEC1(exp, exp)
VEC1(tanh, tanh)
VEC1(cosh, cosh)
VEC1(sin, sin)
VEC1(cos, cos)
VEC1(sqrt, sqrt)
void bsam_vatan2(const double *y, const double *x, double *out, int64_t n) {
  for (int64_t i = 0; i < n; ++i) out[i] = atan2(y[i], x[i]);
}
void bsam_vhypot(const double *x, const double *y, double *out, int64_t n) {
  for (int64_t i = 0; i < n; ++i) out[i] = hypot(x[i], y[i]);
}

/* ---------------------------------------------------------------------- */
typedef struct {
  double box[4];     /* minx miny maxx maxy */
  int left, right;   /* 0 = leaf (node ids are 1-based like the reference) */
  int first, last;   /* segment range, 1-based inclusive */
} Node;

typedef struct {
  int ns;            /* number of segments = npoints - 1 */
  double *a, *e, *len2;  /* a(j,:), e(j,:) interleaved [2*ns]; len2[ns] */
  double *v;         /* vertices [2*npoints] */
  Node *nodes;
  int nnodes, cap;
} Starfish;

static int build_node(Starfish *g, int first, int last) {
  if (g->nnodes == g->cap) {
    g->cap = g->cap ? 2 * g->cap : 256;
    g->nodes = (Node *)realloc(g->nodes, sizeof(Node) * g->cap);
  }
  const int id = ++g->nnodes;  /* 1-based */
  Node *nd = &g->nodes[id - 1];
  double mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
  /* box over a(first:last,:) and b(first:last,:) = v(2:end): the vertices */
  for (int j = first; j <= last; ++j) {
    const double ax = g->v[2 * (j - 1)], ay = g->v[2 * (j - 1) + 1];
    const double bx = g->v[2 * j], by = g->v[2 * j + 1];
    if (ax < mnx) mnx = ax; if (bx < mnx) mnx = bx;
    if (ay < mny) mny = ay; if (by < mny) mny = by;
    if (ax > mxx) mxx = ax; if (bx > mxx) mxx = bx;
    if (ay > mxy) mxy = ay; if (by > mxy) mxy = by;
  }
  nd->box[0] = mnx; nd->box[1] = mny; nd->box[2] = mxx; nd->box[3] = mxy;
  nd->left = nd->right = 0;
  nd->first = first; nd->last = last;
  if (last - first > 15) {
    const int mid = (first + last) / 2;
    const int l = build_node(g, first, mid);
    const int r = build_node(g, mid + 1, last);
    g->nodes[id - 1].left = l;
    g->nodes[id - 1].right = r;
  }
  return id;
}

/* Polygon of n points with r(theta) = s0*(s1 + s2*sin(k*theta + th0)),
   theta = linspace(0, 2*pi, n), last vertex = first.  The reference's
   starfish is s0 = 0.9, s1 = 1.2, s2 = 0.7, k = 5, th0 = 0. */
void *bsam_starfish_new(int n, double s0, double s1, double s2, double k, double th0) {
  Starfish *g = (Starfish *)calloc(1, sizeof(Starfish));
  g->ns = n - 1;
  g->v = (double *)malloc(sizeof(double) * 2 * n);
  const double twopi = 2 * M_PI;
  for (int i = 0; i < n; ++i) {
    /* linspace(0, 2*pi, n): d1 + (i*(d2-d1))/(n-1), last = d2 */
    double th = (i == n - 1) ? twopi : ((double)i * twopi) / (double)(n - 1);
    double arg = (th0 == 0.0) ? k * th : k * th + th0;
    double r = s0 * (s1 + s2 * sin(arg));
    g->v[2 * i] = r * cos(th);
    g->v[2 * i + 1] = r * sin(th);
  }
  g->v[2 * (n - 1)] = g->v[0];
  g->v[2 * (n - 1) + 1] = g->v[1];
  g->a = (double *)malloc(sizeof(double) * 2 * g->ns);
  g->e = (double *)malloc(sizeof(double) * 2 * g->ns);
  g->len2 = (double *)malloc(sizeof(double) * g->ns);
  for (int j = 0; j < g->ns; ++j) {
    g->a[2 * j] = g->v[2 * j];
    g->a[2 * j + 1] = g->v[2 * j + 1];
    g->e[2 * j] = g->v[2 * (j + 1)] - g->v[2 * j];
    g->e[2 * j + 1] = g->v[2 * (j + 1) + 1] - g->v[2 * j + 1];
    g->len2[j] = g->e[2 * j] * g->e[2 * j] + g->e[2 * j + 1] * g->e[2 * j + 1];
  }
  build_node(g, 1, g->ns);
  return g;
}

void bsam_starfish_free(void *p) {
  Starfish *g = (Starfish *)p;
  if (!g) return;
  free(g->v); free(g->a); free(g->e); free(g->len2); free(g->nodes); free(g);
}

int bsam_starfish_nvert(void *p) { return ((Starfish *)p)->ns + 1; }
void bsam_starfish_vertices(void *p, double *out) {
  Starfish *g = (Starfish *)p;
  for (int i = 0; i < 2 * (g->ns + 1); ++i) out[i] = g->v[i];
}

static double box_lb(const Node *nd, double x, double y) {
  const double *bb = nd->box;
  const double dx = fmax(fmax(bb[0] - x, 0.0), x - bb[2]);
  const double dy = fmax(fmax(bb[1] - y, 0.0), y - bb[3]);
  return dx * dx + dy * dy;
}

static inline double seg_d2(const Starfish *g, int j, double x, double y) {
  const double ax = g->a[2 * (j - 1)], ay = g->a[2 * (j - 1) + 1];
  const double ex = g->e[2 * (j - 1)], ey = g->e[2 * (j - 1) + 1];
  double t = ((x - ax) * ex + (y - ay) * ey) / g->len2[j - 1];
  t = fmax(0.0, fmin(1.0, t));
  const double px = (x - ax) - t * ex, py = (y - ay) - t * ey;
  return px * px + py * py;
}

/* The tree search of ddStarfishGeometry.m: a node is entered when its box's
   squared distance is within best + 64 eps.  The result is the minimum over
   every segment whose leaf is entered, and the leaf of the nearest segment
   is always entered, so neither the order in which children are tried nor a
   starting bound that is itself some segment's distance changes the result,
   only how much is pruned: the nearer child goes first, and *arg returns
   the segment that gave the minimum. */
static void visit(const Starfish *g, int id, double lb, double x, double y, double *best, int *arg) {
  if (!(lb <= *best + 64 * DBL_EPSILON)) return;
  const Node *nd = &g->nodes[id - 1];
  if (nd->left != 0) {
    const double ll = box_lb(&g->nodes[nd->left - 1], x, y), lr = box_lb(&g->nodes[nd->right - 1], x, y);
    if (ll < lr) {
      visit(g, nd->left, ll, x, y, best, arg);
      visit(g, nd->right, lr, x, y, best, arg);
    } else {
      visit(g, nd->right, lr, x, y, best, arg);
      visit(g, nd->left, ll, x, y, best, arg);
    }
    return;
  }
  double local = *best;
  int a = *arg;
  for (int j = nd->first; j <= nd->last; ++j) {
    const double dd = seg_d2(g, j, x, y);
    if (dd < local) { local = dd; a = j; }
  }
  *best = local;
  *arg = a;
}

/* Signed distance, positive inside (ddStarfishGeometry.m:140-177).  Points
   are visited in order and each search starts from the smaller of the
   distance to the first vertex of the segment its polar angle falls in and
   the distance to the previous point's nearest segment: on grid-ordered
   samples that bound is tight and prunes most of the tree. */
static void distance_range(const Starfish *g, const double *X, const double *Y, double *d, int64_t n) {
  const double twopi = 2 * M_PI;
  const int ns = g->ns;
  int prev = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double x = X[i], y = Y[i];
    double ang = atan2(y, x);
    ang = ang - floor(ang / twopi) * twopi;      /* mod(atan2(y,x), 2*pi) */
    int seg = (int)floor(ang * ns / twopi) + 1;
    if (seg > ns) seg = ns;
    const double ax = g->a[2 * (seg - 1)], ay = g->a[2 * (seg - 1) + 1];
    double best = (x - ax) * (x - ax) + (y - ay) * (y - ay);
    int arg = seg;
    if (prev > 0) {
      const double dp = seg_d2(g, prev, x, y);
      if (dp < best) { best = dp; arg = prev; }
    }
    visit(g, 1, box_lb(&g->nodes[0], x, y), x, y, &best, &arg);
    prev = arg;
    const double ux = cos(ang), uy = sin(ang);
    const double ex = g->e[2 * (seg - 1)], ey = g->e[2 * (seg - 1) + 1];
    const double radius = (ax * ey - ay * ex) / (ux * ey - uy * ex);
    const double s = (hypot(x, y) > radius) ? -1.0 : 1.0;
    d[i] = s * sqrt(best);
  }
}

void bsam_starfish_distance(void *p, const double *X, const double *Y, double *d, int64_t n) {
  distance_range((const Starfish *)p, X, Y, d, n);
}

/* The same distances on up to `threads` host threads, each over a
   contiguous range of the points (its own warm-start chain).  A point's
   result does not depend on the other points, so any split gives the same
   bits; small calls run on the calling thread. */
typedef struct {
  const Starfish *g;
  const double *X, *Y;
  double *d;
  int64_t n;
} DistJob;

static void *distance_job(void *a) {
  const DistJob *j = (const DistJob *)a;
  distance_range(j->g, j->X, j->Y, j->d, j->n);
  return NULL;
}

void bsam_starfish_distance_mt(void *p, const double *X, const double *Y, double *d, int64_t n, int threads) {
  enum { kMaxThreads = 64, kMinPerThread = 2048 };
  if (threads > kMaxThreads) threads = kMaxThreads;
  if (threads > n / kMinPerThread) threads = (int)(n / kMinPerThread);
  if (threads <= 1) {
    distance_range((const Starfish *)p, X, Y, d, n);
    return;
  }
  pthread_t tid[kMaxThreads];
  DistJob job[kMaxThreads];
  int started[kMaxThreads];
  for (int t = 0; t < threads; ++t) {
    const int64_t lo = n * t / threads, hi = n * (t + 1) / threads;
    job[t].g = (const Starfish *)p;
    job[t].X = X + lo;
    job[t].Y = Y + lo;
    job[t].d = d + lo;
    job[t].n = hi - lo;
    /* thread 0's range runs on the calling thread; a range whose thread
       cannot be started runs there too */
    started[t] = t > 0 && pthread_create(&tid[t], NULL, distance_job, &job[t]) == 0;
  }
  for (int t = 0; t < threads; ++t)
    if (!started[t]) distance_job(&job[t]);
  for (int t = 1; t < threads; ++t)
    if (started[t]) pthread_join(tid[t], NULL);
}

/* The O(n) parts of bsam_starfish_distance for a device minimum: per point
   the starting candidate (squared distance to the first vertex of the
   segment the polar angle falls in) and the sign (+1 inside, -1 outside). */
void bsam_starfish_init_sign(void *p, const double *X, const double *Y, double *init, double *sign, int64_t n) {
  const Starfish *g = (const Starfish *)p;
  const double twopi = 2 * M_PI;
  const int ns = g->ns;
  for (int64_t i = 0; i < n; ++i) {
    const double x = X[i], y = Y[i];
    double ang = atan2(y, x);
    ang = ang - floor(ang / twopi) * twopi;
    int seg = (int)floor(ang * ns / twopi) + 1;
    if (seg > ns) seg = ns;
    const double ax = g->a[2 * (seg - 1)], ay = g->a[2 * (seg - 1) + 1];
    init[i] = (x - ax) * (x - ax) + (y - ay) * (y - ay);
    const double ux = cos(ang), uy = sin(ang);
    const double ex = g->e[2 * (seg - 1)], ey = g->e[2 * (seg - 1) + 1];
    const double radius = (ax * ey - ay * ex) / (ux * ey - uy * ex);
    sign[i] = (hypot(x, y) > radius) ? -1.0 : 1.0;
  }
}
