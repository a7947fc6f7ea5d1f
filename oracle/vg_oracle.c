/* CPU oracle for the VortonSim velocity-from-vorticity step.
 *
 * TEST INFRASTRUCTURE ONLY (see vg_oracle.h).  A plain-C restatement of the
 * reference's algorithms, following the float operation order of the
 * reference's C++ (which the compiler would otherwise be free to fuse), so
 * results are bit-identical to the reference built with -ffp-contract=off.
 * Reference paths are relative to Samples/MjgIntelFluidDemo_Part20.
 */
#include "vg_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI_F 3.1415926535897932384626433832795f

static float maxf_(float a, float b) { return a > b ? a : b; } /* Max2 (Core/Utility/macros.h:64) */
static float minf_(float a, float b) { return a < b ? a : b; } /* Min2 (Core/Utility/macros.h:61) */
static float clampf_(float x, float lo, float hi) { return minf_(maxf_(x, lo), hi); }

/* finvsqrtf (Core/Math/math.h:206-216): Lomont's magic-constant estimate
 * 0x5f3759df - (i >> 1) refined by one Newton step. */
float vgo_finvsqrtf(float v) {
  int32_t i;
  memcpy(&i, &v, 4);
  i = 0x5f3759df - (i >> 1);
  float y;
  memcpy(&y, &i, 4);
  const float f = 1.5f;
  const float x = v * 0.5f;
  y = y * (f - (x * y * y));
  return y;
}

/* ------------------------------------------------------------------ geometry */

/* PrecomputeSpacing (uniformGrid.h:794-809). */
void vgo_precompute_spacing(vgo_geom* g) {
  for (int a = 0; a < 3; ++a) g->cell[a] = g->ext[a] / (float)(g->np[a] - 1);
  g->cpe[0] = (float)(g->np[0] - 1) / g->ext[0];
  g->cpe[1] = (float)(g->np[1] - 1) / g->ext[1];
  g->cpe[2] = (0.0f == g->ext[2]) ? 1.0f / FLT_MIN : (float)(g->np[2] - 1) / g->ext[2];
}

/* NearestPowerOfTwo (Core/Math/math.h:149-175). */
static size_t nearest_pow2(size_t v) {
  if (v == 0) return 1;
  --v;
  unsigned shift = 0;
  while ((v >> shift) != 0) ++shift;
  return (size_t)(1U << shift);
}

/* DefineShape (uniformGrid.h:259-322). */
void vgo_define_shape(size_t n, const float vmin[3], const float vmax[3], int pow2, vgo_geom* g) {
  memset(g, 0, sizeof(*g));
  if (n == 0) return;
  const float nudge = 1.0f + FLT_EPSILON;
  float eff[3];
  int dims = 3;
  for (int a = 0; a < 3; ++a) {
    g->mn[a] = vmin[a];
    g->ext[a] = (vmax[a] - vmin[a]) * nudge;
    eff[a] = g->ext[a];
  }
  for (int a = 0; a < 3; ++a) {
    if (0.0f == eff[a]) {
      eff[a] = 1.0f;
      g->ext[a] = 0.0f;
      --dims;
    }
  }
  const float volume = eff[0] * eff[1] * eff[2];
  const float inv_cell = powf(volume / (float)n, -1.0f / (float)dims);
  size_t nc[3];
  for (int a = 0; a < 3; ++a) {
    size_t c = (size_t)(g->ext[a] * inv_cell + 0.5f);
    nc[a] = c > 1 ? c : 1;
  }
  if (pow2)
    for (int a = 0; a < 3; ++a) nc[a] = nearest_pow2(nc[a]);
  while (nc[0] * nc[1] * nc[2] >= n * 8)
    for (int a = 0; a < 3; ++a) nc[a] = nc[a] / 2 > 1 ? nc[a] / 2 : 1;
  for (int a = 0; a < 3; ++a) g->np[a] = (unsigned)(nc[a] + 1);
  vgo_precompute_spacing(g);
}

/* Decimate (uniformGrid.h:398-412). */
void vgo_decimate(const vgo_geom* src, unsigned dec, vgo_geom* dst) {
  vgo_geom d = *src;
  for (int a = 0; a < 3; ++a) {
    d.np[a] = (src->np[a] - 1) / dec + 1;
    if (dec > 1 && d.np[a] < 2) d.np[a] = 2;
  }
  vgo_precompute_spacing(&d);
  *dst = d;
}

/* IndicesOfPosition (uniformGrid.h:536-574): FP32 (p - min) * cellsPerExtent,
 * truncated toward zero (x87 fistp under a truncating control word). */
void vgo_indices_of_position(const vgo_geom* g, const float p[3], unsigned idx[3]) {
  for (int a = 0; a < 3; ++a) {
    const float rel = p[a] - g->mn[a];
    const float v = rel * g->cpe[a];
    idx[a] = (unsigned)(int)v;
  }
}

/* OffsetOfPosition (uniformGrid.h:645-651). */
unsigned vgo_offset_of_position(const vgo_geom* g, const float p[3]) {
  unsigned i[3];
  vgo_indices_of_position(g, p, i);
  return i[0] + g->np[0] * (i[1] + g->np[1] * i[2]);
}

void vgo_indices_batch(const vgo_geom* g, const float* pos, size_t n, unsigned* idx3, unsigned* offset) {
  for (size_t k = 0; k < n; ++k) {
    vgo_indices_of_position(g, pos + 3 * k, idx3 + 3 * k);
    offset[k] = vgo_offset_of_position(g, pos + 3 * k);
  }
}

static size_t capacity(const vgo_geom* g) { return (size_t)g->np[0] * g->np[1] * g->np[2]; }

/* Particles::PartitionParticles (Particles/particle.cpp:398-437), as called by
 * VortonSim::PartitionVortons (VortonFluid/vortonSim.cpp:3578-3607): walking
 * the particles in index order, each index is appended to the list of the
 * grid point OffsetOfPosition names, so every list is in ascending index
 * order.  Lists are returned flattened: items[start[c] .. start[c+1]) for
 * point c.  A particle whose indices fall outside the points (undefined
 * behaviour in the reference) or whose position is not finite goes to the
 * extra list `points`; start has points + 2 entries. */
void vgo_partition(const vgo_geom* g, const float* pos, size_t n, unsigned* start, unsigned* items) {
  const size_t pts = capacity(g);
  size_t c;
  unsigned* fill;
  for (c = 0; c < pts + 2; ++c) start[c] = 0;
  unsigned* cell = (unsigned*)malloc(n * sizeof(unsigned) + 1);
  for (size_t k = 0; k < n; ++k) {
    const float* p = pos + 3 * k;
    unsigned i[3];
    vgo_indices_of_position(g, p, i);
    size_t off = i[0] + (size_t)g->np[0] * (i[1] + (size_t)g->np[1] * i[2]);
    if (i[0] >= g->np[0] || i[1] >= g->np[1] || i[2] >= g->np[2] || off >= pts || p[0] != p[0] || p[1] != p[1] ||
        p[2] != p[2])
      off = pts;
    cell[k] = (unsigned)off;
    start[off + 1]++;
  }
  for (c = 0; c < pts + 1; ++c) start[c + 1] += start[c];
  fill = (unsigned*)malloc((pts + 1) * sizeof(unsigned));
  for (c = 0; c < pts + 1; ++c) fill[c] = start[c];
  for (size_t k = 0; k < n; ++k) items[fill[cell[k]]++] = (unsigned)k;
  free(fill);
  free(cell);
}

/* NestedGrid::Initialize + PrecomputeDecimations (nestedGrid.h:69-85, 355-391):
 * layer 0 copies g; each parent decimates its child by 2 until the child has
 * at most 8 points.  decim3[3l..3l+2] = child cells / parent cells (l >= 1). */
int vgo_nested_shape(const vgo_geom* g, vgo_geom* layers, unsigned* decim3) {
  int depth = 0;
  vgo_decimate(g, 1, &layers[depth++]);
  while (capacity(&layers[depth - 1]) > 8 && depth < VGO_MAX_LAYERS) {
    vgo_decimate(&layers[depth - 1], 2, &layers[depth]);
    ++depth;
  }
  decim3[0] = decim3[1] = decim3[2] = 0;
  for (int l = 1; l < depth; ++l)
    for (int a = 0; a < 3; ++a) decim3[3 * l + a] = (layers[l - 1].np[a] - 1) / (layers[l].np[a] - 1);
  return depth;
}

/* PclOpFindBoundingBox::FindBoundingBox serial form (pclOpFindBoundingBox.cpp:115-136). */
void vgo_bbox(const float* pos, size_t n, float mn[3], float mx[3]) {
  for (int a = 0; a < 3; ++a) {
    mn[a] = FLT_MAX;
    mx[a] = -FLT_MAX;
  }
  for (size_t k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) {
      mn[a] = minf_(mn[a], pos[3 * k + a]);
      mx[a] = maxf_(mx[a], pos[3 * k + a]);
    }
}

/* PclOpVortonSim::Operate's box -> VortonSim::UpdateBoundingBox(final)
 * (pclOpVortonSim.cpp:51-71, vortonSim.cpp:1027-1096): vorton AABB, joined
 * with the extra box (or the first vorton), padded by 3 radii, then
 * DefineShape(n, ..., pow2). */
void vgo_step_geometry(const float* pos, size_t n, float radius, const float* extra_min, const float* extra_max,
                       vgo_geom* g) {
  float mn[3], mx[3];
  vgo_bbox(pos, n, mn, mx);
  const float* emin = (extra_min && extra_max) ? extra_min : pos;
  const float* emax = (extra_min && extra_max) ? extra_max : pos;
  for (int a = 0; a < 3; ++a) {
    mn[a] = minf_(mn[a], emin[a]);
    mx[a] = maxf_(mx[a], emax[a]);
  }
  const float margin = (1.0f + 2.0f) * radius;
  for (int a = 0; a < 3; ++a) {
    const float d = mx[a] - mn[a];
    mn[a] -= 0.0f * d; /* expansionFactor 0 (vortonSim.cpp:1068-1074) */
    mx[a] += 0.0f * d;
    mn[a] -= margin * 1.0f;
    mx[a] += margin * 1.0f;
  }
  vgo_define_shape(n, mn, mx, 1, g);
}

/* ------------------------------------------------------------- vorton laws */

static const float kTwoThirds = 2.0f / 3.0f; /* vorton.h:92 */

/* VORTON_ACCUMULATE_VELOCITY_private (vorton.h:161-179). */
static void accum_velocity(float acc[3], const float q[3], const float p[3], const float w[3], float size, float sr,
                           float sc) {
  const float d0 = q[0] - p[0], d1 = q[1] - p[1], d2 = q[2] - p[2];
  const float radius = size * 0.5f * sr;
  const float r2 = radius * radius;
  const float dist2 = d0 * d0 + d1 * d1 + d2 * d2;
  const float law = (dist2 < r2) ? (1.0f / (r2 * radius)) : (vgo_finvsqrtf(dist2) / dist2);
  const float s = kTwoThirds * r2 * radius;
  const float a0 = w[0] * s, a1 = w[1] * s, a2 = w[2] * s;
  const float b0 = d0 * law, b1 = d1 * law, b2 = d2 * law;
  const float c0 = a1 * b2 - a2 * b1, c1 = a2 * b0 - a0 * b2, c2 = a0 * b1 - a1 * b0;
  acc[0] += c0 * sc;
  acc[1] += c1 * sc;
  acc[2] += c2 * sc;
}

/* VORTON_ACCUMULATE_VECTOR_POTENTIAL_private (vorton.h:118-136). */
static void accum_vecpot(float acc[3], const float q[3], const float p[3], const float w[3], float size, float sr,
                         float sc) {
  const float d0 = q[0] - p[0], d1 = q[1] - p[1], d2 = q[2] - p[2];
  const float radius = size * 0.5f * sr;
  const float r2 = radius * radius;
  const float dist2 = d0 * d0 + d1 * d1 + d2 * d2;
  const float law = (dist2 < r2) ? (dist2 / (r2 * radius)) : vgo_finvsqrtf(dist2);
  const float s = kTwoThirds * r2 * radius;
  acc[0] += ((w[0] * s) * law) * sc;
  acc[1] += ((w[1] * s) * law) * sc;
  acc[2] += ((w[2] * s) * law) * sc;
}

static void accum(int kind, float acc[3], const float q[3], const float p[3], const float w[3], float size, float sr,
                  float sc) {
  if (kind == 0)
    accum_velocity(acc, q, p, w, size, sr, sc);
  else
    accum_vecpot(acc, q, p, w, size, sr, sc);
}

void vgo_direct(int kind, const float* pos, const float* angvel, const float* size, size_t n, const float* q,
                size_t m, float sr, float sc, float* out) {
  for (size_t j = 0; j < m; ++j) {
    float acc[3] = {0.0f, 0.0f, 0.0f};
    for (size_t i = 0; i < n; ++i) accum(kind, acc, q + 3 * j, pos + 3 * i, angvel + 3 * i, size[i], sr, sc);
    memcpy(out + 3 * j, acc, sizeof(acc));
  }
}

/* The same mollified laws in FP64 with an exact 1/sqrt: the strict oracle. */
void vgo_direct_f64(int kind, const float* pos, const float* angvel, const float* size, size_t n, const float* q,
                    size_t m, float sr, float sc, double* out) {
  for (size_t j = 0; j < m; ++j) {
    double acc[3] = {0, 0, 0};
    for (size_t i = 0; i < n; ++i) {
      const double d0 = (double)q[3 * j] - pos[3 * i], d1 = (double)q[3 * j + 1] - pos[3 * i + 1],
                   d2 = (double)q[3 * j + 2] - pos[3 * i + 2];
      const double radius = (double)size[i] * 0.5 * sr;
      const double r2 = radius * radius;
      const double dist2 = d0 * d0 + d1 * d1 + d2 * d2;
      const double s = (2.0 / 3.0) * r2 * radius * sc;
      const double w0 = angvel[3 * i] * s, w1 = angvel[3 * i + 1] * s, w2 = angvel[3 * i + 2] * s;
      if (kind == 0) {
        const double law = dist2 < r2 ? 1.0 / (r2 * radius) : 1.0 / (sqrt(dist2) * dist2);
        acc[0] += (w1 * d2 - w2 * d1) * law;
        acc[1] += (w2 * d0 - w0 * d2) * law;
        acc[2] += (w0 * d1 - w1 * d0) * law;
      } else {
        const double law = dist2 < r2 ? dist2 / (r2 * radius) : 1.0 / sqrt(dist2);
        acc[0] += w0 * law;
        acc[1] += w1 * law;
        acc[2] += w2 * law;
      }
    }
    out[3 * j] = acc[0];
    out[3 * j + 1] = acc[1];
    out[3 * j + 2] = acc[2];
  }
}

/* ------------------------------------------------------------ influence tree */

typedef struct {
  int depth;
  vgo_geom layer[VGO_MAX_LAYERS];
  unsigned decim[3 * VGO_MAX_LAYERS];
  size_t base[VGO_MAX_LAYERS]; /* first point of each layer in sv */
  float* sv;                   /* 7 floats per point: pos, angvel, size */
} tree_t;

static float vort_mag(const float w[3]) {
  /* GetVorticity().Magnitude(): sqrtf(Mag2(angvel * 2)) (vorton.h:316-320, vec3.h:415-418) */
  const float a = w[0] * 2.0f, b = w[1] * 2.0f, c = w[2] * 2.0f;
  return sqrtf(a * a + b * b + c * c);
}

static void tree_build(tree_t* t, const float* pos, const float* angvel, const float* size, size_t n,
                       const vgo_geom* g) {
  t->depth = vgo_nested_shape(g, t->layer, t->decim);
  size_t total = 0;
  for (int l = 0; l < t->depth; ++l) {
    t->base[l] = total;
    total += capacity(&t->layer[l]);
  }
  t->sv = (float*)calloc(total * 7, sizeof(float));
  /* MakeBaseVortonGrid (vortonSim.cpp:1192-1321). */
  const vgo_geom* leaf = &t->layer[0];
  const size_t nleaf = capacity(leaf);
  float* aux = (float*)malloc(nleaf * sizeof(float));
  for (size_t k = 0; k < nleaf; ++k) aux[k] = FLT_MIN; /* VortonClusterAux (vortonClusterAux.h:71) */
  for (size_t i = 0; i < n; ++i) {
    const unsigned off = vgo_offset_of_position(leaf, pos + 3 * i);
    float* c = t->sv + 7 * (t->base[0] + off);
    const float mag = vort_mag(angvel + 3 * i);
    c[0] += pos[3 * i] * mag;
    c[1] += pos[3 * i + 1] * mag;
    c[2] += pos[3 * i + 2] * mag;
    c[3] += angvel[3 * i];
    c[4] += angvel[3 * i + 1];
    c[5] += angvel[3 * i + 2];
    c[6] = size[i];
    aux[off] += mag;
  }
  for (size_t k = 0; k < nleaf; ++k) {
    if (aux[k] != FLT_MIN) {
      float* c = t->sv + 7 * (t->base[0] + k);
      const float r = 1.0f / aux[k];
      c[0] *= r;
      c[1] *= r;
      c[2] *= r;
    }
  }
  free(aux);
  /* AggregateClusters (vortonSim.cpp:1337-1569). */
  for (int l = 1; l < t->depth; ++l) {
    const vgo_geom* P = &t->layer[l];
    const vgo_geom* C = &t->layer[l - 1];
    const unsigned* d = t->decim + 3 * l;
    for (unsigned pz = 0; pz < P->np[2] - 1; ++pz)
      for (unsigned py = 0; py < P->np[1] - 1; ++py)
        for (unsigned px = 0; px < P->np[0] - 1; ++px) {
          float* p = t->sv + 7 * (t->base[l] + px + P->np[0] * (py + P->np[1] * pz));
          float a = FLT_MIN;
          for (unsigned iz = 0; iz < d[2]; ++iz)
            for (unsigned iy = 0; iy < d[1]; ++iy)
              for (unsigned ix = 0; ix < d[0]; ++ix) {
                const unsigned cx = px * d[0] + ix, cy = py * d[1] + iy, cz = pz * d[2] + iz;
                const float* c = t->sv + 7 * (t->base[l - 1] + cx + C->np[0] * (cy + C->np[1] * cz));
                const float mag = vort_mag(c + 3);
                p[0] += c[0] * mag;
                p[1] += c[1] * mag;
                p[2] += c[2] * mag;
                p[3] += c[3];
                p[4] += c[4];
                p[5] += c[5];
                a += mag;
                if (c[6] != 0.0f) p[6] = c[6];
              }
          const float r = 1.0f / a;
          p[0] *= r;
          p[1] *= r;
          p[2] *= r;
        }
  }
}

size_t vgo_influence_tree(const float* pos, const float* angvel, const float* size, size_t n, const vgo_geom* g,
                          float* out7) {
  tree_t t;
  if (!out7) {
    vgo_geom layers[VGO_MAX_LAYERS];
    unsigned dec[3 * VGO_MAX_LAYERS];
    const int depth = vgo_nested_shape(g, layers, dec);
    size_t total = 0;
    for (int l = 0; l < depth; ++l) total += capacity(&layers[l]);
    return total;
  }
  tree_build(&t, pos, angvel, size, n, g);
  const size_t total = t.base[t.depth - 1] + capacity(&t.layer[t.depth - 1]);
  memcpy(out7, t.sv, total * 7 * sizeof(float));
  free(t.sv);
  return total;
}

/* ComputeVelocity_Tree / ComputeVectorPotential_Tree (vortonSim.cpp:1650-1905):
 * open the child cell containing q (within 1e-4 cell spacings) while the
 * layer is above the leaf's parent; otherwise add the child supervorton. */
static void tree_eval(const tree_t* t, int kind, const float q[3], const unsigned idx[3], int layer, float sr,
                      float sc, float acc_out[3]) {
  const vgo_geom* C = &t->layer[layer - 1];
  const unsigned* d = t->decim + 3 * layer;
  const unsigned cmin[3] = {idx[0] * d[0], idx[1] * d[1], idx[2] * d[2]};
  const float margin_factor = 0.0001f;
  float margin[3] = {margin_factor * C->cell[0], margin_factor * C->cell[1], margin_factor * C->cell[2]};
  margin[0] = margin[0] + 0.0f;
  margin[1] = margin[1] + 0.0f;
  margin[2] = margin[2] + (0.0f == C->cell[2] ? FLT_MIN : 0.0f);
  float acc[3] = {0.0f, 0.0f, 0.0f};
  for (unsigned iz = 0; iz < d[2]; ++iz) {
    unsigned ch[3];
    ch[2] = cmin[2] + iz;
    const float mnz = C->mn[2] + (float)ch[2] * C->cell[2];
    const float mxz = C->mn[2] + (float)(ch[2] + 1) * C->cell[2];
    for (unsigned iy = 0; iy < d[1]; ++iy) {
      ch[1] = cmin[1] + iy;
      const float mny = C->mn[1] + (float)ch[1] * C->cell[1];
      const float mxy = C->mn[1] + (float)(ch[1] + 1) * C->cell[1];
      for (unsigned ix = 0; ix < d[0]; ++ix) {
        ch[0] = cmin[0] + ix;
        const float mnx = C->mn[0] + (float)ch[0] * C->cell[0];
        const float mxx = C->mn[0] + (float)(ch[0] + 1) * C->cell[0];
        if (layer > 1 && q[0] >= mnx - margin[0] && q[1] >= mny - margin[1] && q[2] >= mnz - margin[2] &&
            q[0] < mxx + margin[0] && q[1] < mxy + margin[1] && q[2] < mxz + margin[2]) {
          float sub[3];
          tree_eval(t, kind, q, ch, layer - 1, sr, sc, sub);
          acc[0] += sub[0];
          acc[1] += sub[1];
          acc[2] += sub[2];
        } else {
          const float* s = t->sv + 7 * (t->base[layer - 1] + ch[0] + C->np[0] * (ch[1] + C->np[1] * ch[2]));
          accum(kind, acc, q, s, s + 3, s[6], sr, sc);
        }
      }
    }
  }
  memcpy(acc_out, acc, sizeof(acc));
}

static void tree_query(const tree_t* t, int kind, const float* pos, const float* angvel, const float* size, size_t n,
                       const float q[3], float sr, float sc, float out[3]) {
  static const unsigned zeros[3] = {0, 0, 0};
  if (t->depth > 1) {
    tree_eval(t, kind, q, zeros, t->depth - 1, sr, sc, out);
  } else {
    float acc[3] = {0, 0, 0};
    for (size_t i = 0; i < n; ++i) accum(kind, acc, q, pos + 3 * i, angvel + 3 * i, size[i], sr, sc);
    memcpy(out, acc, sizeof(acc));
  }
}

/* The number of pair laws the walk of tree_eval evaluates for query q: the
 * same open test (vortonSim.cpp:1707-1719), counting instead of adding. */
static size_t tree_count(const vgo_geom* layers, const unsigned* decim, const float q[3], const unsigned idx[3],
                         int layer) {
  const vgo_geom* C = &layers[layer - 1];
  const unsigned* d = decim + 3 * layer;
  const float margin_factor = 0.0001f;
  float margin[3] = {margin_factor * C->cell[0], margin_factor * C->cell[1], margin_factor * C->cell[2]};
  margin[2] = margin[2] + (0.0f == C->cell[2] ? FLT_MIN : 0.0f);
  size_t count = 0;
  for (unsigned iz = 0; iz < d[2]; ++iz) {
    unsigned ch[3];
    ch[2] = idx[2] * d[2] + iz;
    const float mnz = C->mn[2] + (float)ch[2] * C->cell[2];
    const float mxz = C->mn[2] + (float)(ch[2] + 1) * C->cell[2];
    for (unsigned iy = 0; iy < d[1]; ++iy) {
      ch[1] = idx[1] * d[1] + iy;
      const float mny = C->mn[1] + (float)ch[1] * C->cell[1];
      const float mxy = C->mn[1] + (float)(ch[1] + 1) * C->cell[1];
      for (unsigned ix = 0; ix < d[0]; ++ix) {
        ch[0] = idx[0] * d[0] + ix;
        const float mnx = C->mn[0] + (float)ch[0] * C->cell[0];
        const float mxx = C->mn[0] + (float)(ch[0] + 1) * C->cell[0];
        if (layer > 1 && q[0] >= mnx - margin[0] && q[1] >= mny - margin[1] && q[2] >= mnz - margin[2] &&
            q[0] < mxx + margin[0] && q[1] < mxy + margin[1] && q[2] < mxz + margin[2])
          count += tree_count(layers, decim, q, ch, layer - 1);
        else
          count += 1;
      }
    }
  }
  return count;
}

/* Total pair laws of the treecode walk (ComputeVelocity_Tree from the root)
 * over m queries on the NestedGrid of g: the interaction count behind the
 * treecode's FP32 roofline. */
size_t vgo_tree_interactions(const vgo_geom* g, const float* q, size_t m) {
  vgo_geom layers[VGO_MAX_LAYERS];
  unsigned dec[3 * VGO_MAX_LAYERS];
  static const unsigned zeros[3] = {0, 0, 0};
  const int depth = vgo_nested_shape(g, layers, dec);
  size_t total = 0;
  if (depth < 2) return 0;
  for (size_t j = 0; j < m; ++j) total += tree_count(layers, dec, q + 3 * j, zeros, depth - 1);
  return total;
}

void vgo_tree(int kind, const float* pos, const float* angvel, const float* size, size_t n, const vgo_geom* g,
              const float* q, size_t m, float sr, float sc, float* out) {
  tree_t t;
  tree_build(&t, pos, angvel, size, n, g);
  for (size_t j = 0; j < m; ++j) tree_query(&t, kind, pos, angvel, size, n, q + 3 * j, sr, sc, out + 3 * j);
  free(t.sv);
}

/* -------------------------------------------------------------- grid fields */

/* PopulateVorticityGridFromVortons (vortonSim.cpp:2372-2436) with
 * UniformGrid::Accumulate (uniformGrid.h:1278-1342). */
void vgo_splat(const float* pos, const float* angvel, const float* size, size_t n, const vgo_geom* g, float scale,
               float* grid) {
  memset(grid, 0, capacity(g) * 3 * sizeof(float));
  if (n == 0) return;
  const float radius = size[0] * 0.5f;
  const float cell_volume = g->cell[0] * g->cell[1] * g->cell[2];
  const float four_pi_over3 = (4.0f * PI_F) / 3.0f;
  const float vorton_volume = four_pi_over3 * (radius * radius * radius);
  const float corr = scale * vorton_volume / cell_volume;
  const unsigned nx = g->np[0], nxy = g->np[0] * g->np[1];
  for (size_t i = 0; i < n; ++i) {
    const float* p = pos + 3 * i;
    const float item[3] = {(angvel[3 * i] * 2.0f) * corr, (angvel[3 * i + 1] * 2.0f) * corr,
                           (angvel[3 * i + 2] * 2.0f) * corr};
    unsigned idx[3];
    vgo_indices_of_position(g, p, idx);
    float tw[3], om[3];
    for (int a = 0; a < 3; ++a) {
      const float cmin = g->mn[a] + (float)idx[a] * g->cell[a];
      const float diff = p[a] - cmin;
      tw[a] = clampf_(diff * g->cpe[a], 0.0f, 1.0f);
      om[a] = 1.0f - tw[a];
    }
    const size_t o = idx[0] + (size_t)nx * (idx[1] + (size_t)g->np[1] * idx[2]);
    const size_t offs[8] = {o, o + 1, o + nx, o + nx + 1, o + nxy, o + nxy + 1, o + nxy + nx, o + nxy + nx + 1};
    const float w[8] = {om[0] * om[1] * om[2], tw[0] * om[1] * om[2], om[0] * tw[1] * om[2], tw[0] * tw[1] * om[2],
                        om[0] * om[1] * tw[2], tw[0] * om[1] * tw[2], om[0] * tw[1] * tw[2], tw[0] * tw[1] * tw[2]};
    for (int c = 0; c < 8; ++c)
      for (int a = 0; a < 3; ++a) grid[3 * offs[c] + a] += w[c] * item[a];
  }
}

/* ComputeVectorPotentialAtGridpoints_Slice (vortonSim.cpp:2055-2138) over all
 * z; copy_odd_x reproduces the reference's reuse of the preceding even-x value
 * on odd-x points. */
void vgo_boundary_vecpot(const float* pos, const float* angvel, const float* size, size_t n, const vgo_geom* g,
                         int boundaries_only, int copy_odd_x, float* grid) {
  tree_t t;
  tree_build(&t, pos, angvel, size, n, g);
  const float nudge = 1.0f - 2.0f * FLT_EPSILON;
  const float sp[3] = {g->cell[0] * nudge, g->cell[1] * nudge, g->cell[2] * nudge};
  const unsigned* dims = g->np;
  const unsigned nxy = dims[0] * dims[1];
  const unsigned inc_interior = boundaries_only ? (dims[0] - 1) : 1;
  for (unsigned z = 0; z < dims[2]; ++z) {
    float p[3];
    p[2] = g->mn[2] + (float)z * sp[2];
    const int tb = (0 == z) || (dims[2] - 1 == z);
    for (unsigned y = 0; y < dims[1]; ++y) {
      p[1] = g->mn[1] + (float)y * sp[1];
      const int fb = (0 == y) || (dims[1] - 1 == y);
      const unsigned incx = (tb || fb) ? 1 : inc_interior;
      for (unsigned x = 0; x < dims[0]; x += incx) {
        p[0] = g->mn[0] + (float)x * sp[0];
        const unsigned off = x + y * dims[0] + z * nxy;
        if (!copy_odd_x || 0 == (x & 1))
          tree_query(&t, 1, pos, angvel, size, n, p, 1.0f, 1.0f, grid + 3 * off);
        else
          memcpy(grid + 3 * off, grid + 3 * (off - 1), 3 * sizeof(float));
      }
    }
  }
  free(t.sv);
}

/* StepTowardVectorPoissonSolution, red then black, Dirichlet
 * (uniformGridMath.cpp:1116-1339, 1369-1405): SOR with relaxation 1.72 over
 * x-rows whose (y + z) parity matches the colour, each row swept in +x. */
void vgo_sor(const vgo_geom* g, float* s, const float* lap, int steps) {
  const float* sp = g->cell;
  const float rs[3] = {1.0f / sp[0], 1.0f / sp[1], sp[2] > FLT_EPSILON ? 1.0f / sp[2] : 0.0f};
  const float rs2[3] = {rs[0] * rs[0], rs[1] * rs[1], rs[2] * rs[2]};
  const float H = 0.5f / (rs2[0] + rs2[1] + rs2[2]);
  const size_t nx = g->np[0], ny = g->np[1], nz = g->np[2], nxy = nx * ny;
  const float relax = 1.72f;
  const float omr = 1.0f - relax;
  for (int it = 0; it < steps; ++it) {
    for (unsigned color = 0; color < 2; ++color) {
      for (size_t z = 1; z + 1 < nz; ++z) {
        const size_t yshift = (z % 2 == color) ? 1 : 0;
        for (size_t y = 1 + yshift; y + 1 < ny; y += 2) {
          for (size_t x = 1; x + 1 < nx; ++x) {
            const size_t c = x + nx * y + nxy * z;
            for (int a = 0; a < 3; ++a) {
              const float v = ((s[3 * (c + 1) + a] + s[3 * (c - 1) + a]) * rs2[0] +
                               (s[3 * (c + nx) + a] + s[3 * (c - nx) + a]) * rs2[1] +
                               (s[3 * (c + nxy) + a] + s[3 * (c - nxy) + a]) * rs2[2] - lap[3 * c + a]) *
                              H;
              s[3 * c + a] = omr * s[3 * c + a] + relax * v;
            }
          }
        }
      }
    }
  }
}

/* DownSampleSlice (uniformGrid.h:1453-1585): inject = FASTER_LESS_ACCURATE
 * (copy the cluster's min-corner point); else SLOWER_MORE_ACCURATE (27-point
 * full weighting around it, out-of-range points omitted). */
void vgo_downsample(const vgo_geom* fine, const float* fv, int inject, const vgo_geom* coarse, float* cv) {
  const unsigned cd[3] = {(fine->np[0] - 1) / (coarse->np[0] - 1), (fine->np[1] - 1) / (coarse->np[1] - 1),
                          (fine->np[2] - 1) / (coarse->np[2] - 1)};
  const unsigned fnx = fine->np[0], fnxy = fine->np[0] * fine->np[1];
  for (unsigned z = 0; z < coarse->np[2]; ++z)
    for (unsigned y = 0; y < coarse->np[1]; ++y)
      for (unsigned x = 0; x < coarse->np[0]; ++x) {
        float* o = cv + 3 * (x + coarse->np[0] * (y + coarse->np[1] * z));
        const unsigned mx = x * cd[0], my = y * cd[1], mz = z * cd[2];
        if (inject) {
          const float* f = fv + 3 * (mx + my * fnx + mz * fnxy);
          o[0] = f[0];
          o[1] = f[1];
          o[2] = f[2];
        } else {
          /* USE_ALL_NEIGHBORS (uniformGrid.h:43): 27-point full weighting,
             8/4/2/1 by Manhattan distance, normalised by 64 */
          static const float table[4] = {8.0f, 4.0f, 2.0f, 1.0f};
          const unsigned sh[3] = {cd[0] / 2, cd[1] / 2, cd[2] / 2};
          float acc[3] = {0, 0, 0};
          for (unsigned iz = 0; iz < cd[2] + sh[2]; ++iz) {
            const int s2 = (int)iz - (int)sh[2];
            const unsigned hz = mz + (unsigned)s2;
            if (hz >= fine->np[2]) continue;
            for (unsigned iy = 0; iy < cd[1] + sh[1]; ++iy) {
              const int s1 = (int)iy - (int)sh[1];
              const unsigned hy = my + (unsigned)s1;
              if (hy >= fine->np[1]) continue;
              for (unsigned ix = 0; ix < cd[0] + sh[0]; ++ix) {
                const int s0 = (int)ix - (int)sh[0];
                const unsigned hx = mx + (unsigned)s0;
                if (hx >= fine->np[0]) continue;
                const unsigned md = (unsigned)(abs(s0) + abs(s1) + abs(s2));
                const float* f = fv + 3 * (hx + hy * fnx + hz * fnxy);
                acc[0] += table[md] * f[0];
                acc[1] += table[md] * f[1];
                acc[2] += table[md] * f[2];
              }
            }
          }
          const float r = 1.0f / 64.0f;
          o[0] = acc[0] * r;
          o[1] = acc[1] * r;
          o[2] = acc[2] * r;
        }
      }
}

/* UniformGrid::Interpolate (uniformGrid.h:1117-1148) for a 3-vector field. */
void vgo_interpolate3(const vgo_geom* g, const float* f, const float p[3], float out[3]) {
  unsigned idx[3];
  vgo_indices_of_position(g, p, idx);
  float tw[3], om[3];
  for (int a = 0; a < 3; ++a) {
    const float cmin = g->mn[a] + (float)idx[a] * g->cell[a];
    tw[a] = (p[a] - cmin) * g->cpe[a];
    om[a] = 1.0f - tw[a];
  }
  const size_t nx = g->np[0], nxy = (size_t)g->np[0] * g->np[1];
  const size_t o = idx[0] + nx * (idx[1] + (size_t)g->np[1] * idx[2]);
  for (int a = 0; a < 3; ++a) {
    const float v000 = f[3 * o + a], v100 = f[3 * (o + 1) + a], v010 = f[3 * (o + nx) + a],
                v110 = f[3 * (o + nx + 1) + a], v001 = f[3 * (o + nxy) + a], v101 = f[3 * (o + nxy + 1) + a],
                v011 = f[3 * (o + nxy + nx) + a], v111 = f[3 * (o + nxy + nx + 1) + a];
    out[a] = ((om[0] * v000 + tw[0] * v100) * om[1] + (om[0] * v010 + tw[0] * v110) * tw[1]) * om[2] +
             ((om[0] * v001 + tw[0] * v101) * om[1] + (om[0] * v011 + tw[0] * v111) * tw[1]) * tw[2];
  }
}

/* Interpolate for a field of k floats per point (Mat33: k = 9). */
static void interpolate_k(const vgo_geom* g, const float* f, int k, const float p[3], float* out) {
  unsigned idx[3];
  vgo_indices_of_position(g, p, idx);
  float tw[3], om[3];
  for (int a = 0; a < 3; ++a) {
    const float cmin = g->mn[a] + (float)idx[a] * g->cell[a];
    tw[a] = (p[a] - cmin) * g->cpe[a];
    om[a] = 1.0f - tw[a];
  }
  const size_t nx = g->np[0], nxy = (size_t)g->np[0] * g->np[1];
  const size_t o = idx[0] + nx * (idx[1] + (size_t)g->np[1] * idx[2]);
  for (int a = 0; a < k; ++a) {
    const float v000 = f[k * o + a], v100 = f[k * (o + 1) + a], v010 = f[k * (o + nx) + a],
                v110 = f[k * (o + nx + 1) + a], v001 = f[k * (o + nxy) + a], v101 = f[k * (o + nxy + 1) + a],
                v011 = f[k * (o + nxy + nx) + a], v111 = f[k * (o + nxy + nx + 1) + a];
    out[a] = ((om[0] * v000 + tw[0] * v100) * om[1] + (om[0] * v010 + tw[0] * v110) * tw[1]) * om[2] +
             ((om[0] * v001 + tw[0] * v101) * om[1] + (om[0] * v011 + tw[0] * v111) * tw[1]) * tw[2];
  }
}

/* UpSampleSlice (uniformGrid.h:1637-1700): sample the coarse grid at fine
 * points nudged inward by 2 eps |min| and spacing * (1 - 4 eps). */
void vgo_upsample(const vgo_geom* coarse, const float* cv, const vgo_geom* fine, int interior_only, float* fv) {
  const float pmin[3] = {fine->mn[0] + fabsf(fine->mn[0]) * 2.0f * FLT_EPSILON,
                         fine->mn[1] + fabsf(fine->mn[1]) * 2.0f * FLT_EPSILON,
                         fine->mn[2] + fabsf(fine->mn[2]) * 2.0f * FLT_EPSILON};
  const float shrink = 1.0f - 4.0f * FLT_EPSILON;
  const float sp[3] = {fine->cell[0] * shrink, fine->cell[1] * shrink, fine->cell[2] * shrink};
  unsigned lo[3] = {0, 0, 0}, hi[3] = {fine->np[0], fine->np[1], fine->np[2]};
  if (interior_only) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = 1;
      hi[a] = (fine->np[a] > 1 ? fine->np[a] : 1) - 1;
    }
  }
  for (unsigned z = lo[2]; z < hi[2]; ++z) {
    float p[3];
    p[2] = pmin[2] + (float)z * sp[2];
    for (unsigned y = lo[1]; y < hi[1]; ++y) {
      p[1] = pmin[1] + (float)y * sp[1];
      for (unsigned x = lo[0]; x < hi[0]; ++x) {
        p[0] = pmin[0] + (float)x * sp[0];
        vgo_interpolate3(coarse, cv, p, fv + 3 * (x + fine->np[0] * (y + fine->np[1] * z)));
      }
    }
  }
}

/* The cascade in VortonSim::ComputeVectorPotential (vortonSim.cpp:2539-2571). */
void vgo_cascade(const vgo_geom* g, float* soln, const float* rhs, int steps) {
  vgo_geom L[VGO_MAX_LAYERS];
  unsigned dec[3 * VGO_MAX_LAYERS];
  const int depth = vgo_nested_shape(g, L, dec);
  float* a[VGO_MAX_LAYERS];
  float* b[VGO_MAX_LAYERS];
  for (int l = 0; l < depth; ++l) {
    a[l] = (float*)calloc(capacity(&L[l]) * 3, sizeof(float));
    b[l] = (float*)calloc(capacity(&L[l]) * 3, sizeof(float));
  }
  memcpy(a[0], soln, capacity(g) * 3 * sizeof(float));
  memcpy(b[0], rhs, capacity(g) * 3 * sizeof(float));
  vgo_sor(&L[0], a[0], b[0], steps);
  int max_valid = 0;
  for (int l = 1; l < depth; ++l) {
    unsigned mind = L[l].np[0] < L[l].np[1] ? L[l].np[0] : L[l].np[1];
    if (L[l].np[2] < mind) mind = L[l].np[2];
    if (mind > 2) {
      vgo_downsample(&L[l - 1], b[l - 1], 1, &L[l], b[l]);
      vgo_downsample(&L[l - 1], a[l - 1], 1, &L[l], a[l]);
      vgo_sor(&L[l], a[l], b[l], steps);
    } else {
      max_valid = l - 1;
      break;
    }
  }
  for (int l = max_valid; l >= 1; --l) {
    vgo_upsample(&L[l], a[l], &L[l - 1], 1, a[l - 1]);
    vgo_sor(&L[l - 1], a[l - 1], b[l - 1], steps);
  }
  memcpy(soln, a[0], capacity(g) * 3 * sizeof(float));
  for (int l = 0; l < depth; ++l) {
    free(a[l]);
    free(b[l]);
  }
}

/* ComputeJacobian (uniformGridMath.cpp:304-451): j[3*a + b] = d v_b / d a;
 * central differences inside, one-sided on each boundary face. */
void vgo_jacobian(const vgo_geom* g, const float* v, float* jac) {
  const float* sp = g->cell;
  const float rs[3] = {1.0f / sp[0], 1.0f / sp[1], sp[2] > FLT_EPSILON ? 1.0f / sp[2] : 0.0f};
  const float hrs[3] = {0.5f * rs[0], 0.5f * rs[1], 0.5f * rs[2]};
  const size_t n[3] = {g->np[0], g->np[1], g->np[2]};
  const size_t stride[3] = {1, n[0], n[0] * n[1]};
  for (size_t z = 0; z < n[2]; ++z)
    for (size_t y = 0; y < n[1]; ++y)
      for (size_t x = 0; x < n[0]; ++x) {
        const size_t c = x + stride[1] * y + stride[2] * z;
        const size_t idx[3] = {x, y, z};
        for (int a = 0; a < 3; ++a) {
          size_t hi = c, lo = c;
          float f;
          if (idx[a] == 0) {
            hi = c + stride[a];
            f = rs[a];
          } else if (idx[a] == n[a] - 1) {
            lo = c - stride[a];
            f = rs[a];
          } else {
            hi = c + stride[a];
            lo = c - stride[a];
            f = hrs[a];
          }
          for (int b = 0; b < 3; ++b) jac[9 * c + 3 * a + b] = (v[3 * hi + b] - v[3 * lo + b]) * f;
        }
      }
}

/* ComputeCurlFromJacobian (uniformGridMath.cpp:207-232). */
void vgo_curl_from_jacobian(size_t points, const float* j, float* curl) {
  for (size_t c = 0; c < points; ++c) {
    const float* m = j + 9 * c;
    curl[3 * c] = m[5] - m[7];     /* j.y.z - j.z.y */
    curl[3 * c + 1] = m[6] - m[2]; /* j.z.x - j.x.z */
    curl[3 * c + 2] = m[1] - m[3]; /* j.x.y - j.y.x */
  }
}

/* StretchAndTiltVortons (vortonSim.cpp:2748-2820): interpolate the velocity
 * Jacobian at each vorton, stretchTilt = angvel * J (transpose form),
 * angvel += 0.5 * stretchTilt * dt. */
void vgo_stretch(const float* pos, float* w, size_t n, const vgo_geom* g, const float* jac9, float dt) {
  if (0.0f == g->ext[0] || 0.0f == g->ext[1] || 0.0f == g->ext[2]) return;
  for (size_t i = 0; i < n; ++i) {
    float J[9];
    interpolate_k(g, jac9, 9, pos + 3 * i, J);
    float* a = w + 3 * i;
    const float st[3] = {J[0] * a[0] + J[1] * a[1] + J[2] * a[2], J[3] * a[0] + J[4] * a[1] + J[5] * a[2],
                         J[6] * a[0] + J[7] * a[1] + J[8] * a[2]};
    a[0] += (0.5f * st[0]) * dt;
    a[1] += (0.5f * st[1]) * dt;
    a[2] += (0.5f * st[2]) * dt;
  }
}

/* ---------------------------------------------------------------- PSE */

typedef struct {
  unsigned* start; /* per cell, points layout of g */
  unsigned* count;
  unsigned* items; /* vorton indices, ascending within each cell */
} cells_t;

/* PartitionParticles (particle.cpp:398-437): each vorton's index appended to
 * the list of the cell OffsetOfPosition names, in index order. */
static void cells_build(cells_t* c, const float* pos, size_t n, const vgo_geom* g) {
  const size_t cap = capacity(g);
  c->start = (unsigned*)calloc(cap + 1, sizeof(unsigned));
  c->count = (unsigned*)calloc(cap, sizeof(unsigned));
  c->items = (unsigned*)malloc((n ? n : 1) * sizeof(unsigned));
  unsigned* off = (unsigned*)malloc((n ? n : 1) * sizeof(unsigned));
  for (size_t i = 0; i < n; ++i) {
    off[i] = vgo_offset_of_position(g, pos + 3 * i);
    c->count[off[i]]++;
  }
  for (size_t k = 0; k < cap; ++k) c->start[k + 1] = c->start[k] + c->count[k];
  unsigned* fill = (unsigned*)calloc(cap, sizeof(unsigned));
  for (size_t i = 0; i < n; ++i) c->items[c->start[off[i]] + fill[off[i]]++] = (unsigned)i;
  free(fill);
  free(off);
}

static void cells_free(cells_t* c) {
  free(c->start);
  free(c->count);
  free(c->items);
}

/* ExchangeVorticityOrMergeVortons without merging (vortonSim.cpp:3616-3669). */
static void exchange(const float* pos, float* w, const float* size, unsigned h, unsigned t, float viscosity,
                     float dt) {
  const float range = 4.0f * size[h];
  const float range2 = range * range;
  const float s0 = pos[3 * h] - pos[3 * t], s1 = pos[3 * h + 1] - pos[3 * t + 1], s2 = pos[3 * h + 2] - pos[3 * t + 2];
  const float dist2 = s0 * s0 + s1 * s1 + s2 * s2;
  const float law = expf(-dist2 / range2);
  const float d[3] = {w[3 * h] - w[3 * t], w[3 * h + 1] - w[3 * t + 1], w[3 * h + 2] - w[3 * t + 2]};
  const float frac = clampf_(2.0f * viscosity * dt * law, -0.5f, 0.5f);
  for (int a = 0; a < 3; ++a) {
    const float e = frac * d[a];
    w[3 * h + a] -= e;
    w[3 * t + a] += e;
  }
}

/* The 7 forward neighbour cells (vortonSim.cpp:3712-3727). */
static void forward_offsets(const vgo_geom* g, size_t off[7]) {
  const size_t nx = g->np[0], nxy = (size_t)g->np[0] * g->np[1];
  off[0] = 1;
  off[1] = nx;
  off[2] = 1 + nx;
  off[3] = nxy;
  off[4] = 1 + nxy;
  off[5] = nx + nxy;
  off[6] = 1 + nx + nxy;
}

/* DiffuseAndDissipateVorticityPSESlice, serial PHASE_BOTH
 * (vortonSim.cpp:3678-3800): in-place pairwise exchange in cell order. */
void vgo_pse_sequential(const float* pos, float* w, const float* size, size_t n, const vgo_geom* g, float viscosity,
                        float dt) {
  cells_t c;
  cells_build(&c, pos, n, g);
  size_t fo[7];
  forward_offsets(g, fo);
  const float diss = viscosity * dt;
  const size_t nx = g->np[0], ny = g->np[1], nz = g->np[2], nxy = nx * ny;
  for (size_t z = 0; z + 1 < nz; ++z)
    for (size_t y = 0; y + 1 < ny; ++y)
      for (size_t x = 0; x + 1 < nx; ++x) {
        const size_t cell = x + y * nx + z * nxy;
        for (unsigned ih = 0; ih < c.count[cell]; ++ih) {
          const unsigned h = c.items[c.start[cell] + ih];
          for (unsigned it = ih + 1; it < c.count[cell]; ++it)
            exchange(pos, w, size, h, c.items[c.start[cell] + it], viscosity, dt);
          for (int k = 0; k < 7; ++k) {
            const size_t nb = cell + fo[k];
            for (unsigned it = 0; it < c.count[nb]; ++it) exchange(pos, w, size, h, c.items[c.start[nb] + it], viscosity, dt);
          }
          for (int a = 0; a < 3; ++a) w[3 * h + a] -= diss * w[3 * h + a];
        }
      }
  cells_free(&c);
}

/* Order-independent form of the same exchange, used by the GPU: every pair
 * the reference visits (same cell, or cells offset by {0,1}^3 in either
 * direction, the "here" cell strictly inside the point range) exchanges
 * using the values from before the step; each vorton whose cell is a "here"
 * cell then dissipates.  Differs from the reference's in-place order by
 * O((2 nu dt)^2) of the vorticity differences. */
void vgo_pse_symmetric(const float* pos, float* w, const float* size, size_t n, const vgo_geom* g, float viscosity,
                       float dt) {
  cells_t c;
  cells_build(&c, pos, n, g);
  float* w0 = (float*)malloc((n ? n : 1) * 3 * sizeof(float));
  memcpy(w0, w, n * 3 * sizeof(float));
  const float diss = viscosity * dt;
  const int nx = (int)g->np[0], ny = (int)g->np[1], nz = (int)g->np[2];
  for (size_t i = 0; i < n; ++i) {
    unsigned id[3];
    vgo_indices_of_position(g, pos + 3 * i, id);
    const int ci[3] = {(int)id[0], (int)id[1], (int)id[2]};
    const int here_ok = ci[0] < nx - 1 && ci[1] < ny - 1 && ci[2] < nz - 1;
    double acc[3] = {0, 0, 0};
    for (int s = -1; s <= 1; s += 2) {
      for (int k = 0; k < 8; ++k) {
        const int d[3] = {s * (k & 1), s * ((k >> 1) & 1), s * ((k >> 2) & 1)};
        if (k == 0 && s == 1) continue; /* same cell handled with s == -1 */
        const int nc[3] = {ci[0] + d[0], ci[1] + d[1], ci[2] + d[2]};
        if (nc[0] < 0 || nc[1] < 0 || nc[2] < 0 || nc[0] >= nx || nc[1] >= ny || nc[2] >= nz) continue;
        /* the pair is visited from the lower cell, which must be a "here" cell */
        const int* lower = (s == 1) ? ci : nc;
        if (!(lower[0] < nx - 1 && lower[1] < ny - 1 && lower[2] < nz - 1)) continue;
        const size_t cell = (size_t)nc[0] + (size_t)nx * ((size_t)nc[1] + (size_t)ny * nc[2]);
        for (unsigned it = 0; it < c.count[cell]; ++it) {
          const unsigned j = c.items[c.start[cell] + it];
          if (j == i) continue;
          /* the range uses the size of the pair's "here" vorton: the one in
             the lower cell, or the lower index within one cell */
          const size_t here = (k == 0) ? (i < j ? i : j) : (s == 1 ? i : j);
          const float range = 4.0f * size[here];
          const float range2 = range * range;
          const float s0 = pos[3 * i] - pos[3 * j], s1 = pos[3 * i + 1] - pos[3 * j + 1], s2 = pos[3 * i + 2] - pos[3 * j + 2];
          const float dist2 = s0 * s0 + s1 * s1 + s2 * s2;
          const float law = expf(-dist2 / range2);
          const float frac = clampf_(2.0f * viscosity * dt * law, -0.5f, 0.5f);
          for (int a = 0; a < 3; ++a) acc[a] += (double)frac * ((double)w0[3 * j + a] - w0[3 * i + a]);
        }
      }
    }
    for (int a = 0; a < 3; ++a) {
      float v = (float)((double)w0[3 * i + a] + acc[a]);
      if (here_ok) v -= diss * v;
      w[3 * i + a] = v;
    }
  }
  free(w0);
  cells_free(&c);
}

/* AssignParticleVelocityFromField_Slice, gain 1 (pclOpAdvect.cpp:42-81). */
void vgo_gather(const vgo_geom* g, const float* velgrid, const float* pos, size_t n, float* vel) {
  for (size_t i = 0; i < n; ++i) vgo_interpolate3(g, velgrid, pos + 3 * i, vel + 3 * i);
}

/* EvolveParticlesSlice (pclOpEvolve.cpp:36-58): pos += vel * dt. */
void vgo_evolve(float* pos, const float* vel, size_t n, float dt) {
  for (size_t i = 0; i < 3 * n; ++i) pos[i] += vel[i] * dt;
}

/* ----------------------------------------------------------- residual norms */

static double relres_impl(const vgo_geom* g, const float* af, const double* ad, const float* b) {
  const size_t nx = g->np[0], ny = g->np[1], nz = g->np[2], nxy = nx * ny;
  const double h2[3] = {1.0 / ((double)g->cell[0] * g->cell[0]), 1.0 / ((double)g->cell[1] * g->cell[1]),
                        1.0 / ((double)g->cell[2] * g->cell[2])};
  double rr = 0, bb = 0;
#define A_(i) (af ? (double)af[i] : ad[i])
  for (size_t z = 1; z + 1 < nz; ++z)
    for (size_t y = 1; y + 1 < ny; ++y)
      for (size_t x = 1; x + 1 < nx; ++x) {
        const size_t c = x + nx * y + nxy * z;
        for (int a = 0; a < 3; ++a) {
          const double ac = A_(3 * c + a);
          const double lap = (A_(3 * (c + 1) + a) + A_(3 * (c - 1) + a) - 2 * ac) * h2[0] +
                             (A_(3 * (c + nx) + a) + A_(3 * (c - nx) + a) - 2 * ac) * h2[1] +
                             (A_(3 * (c + nxy) + a) + A_(3 * (c - nxy) + a) - 2 * ac) * h2[2];
          const double r = (double)b[3 * c + a] - lap;
          rr += r * r;
          bb += (double)b[3 * c + a] * b[3 * c + a];
        }
      }
#undef A_
  return bb > 0 ? sqrt(rr / bb) : sqrt(rr);
}

double vgo_relres_f64(const vgo_geom* g, const float* a, const float* b) { return relres_impl(g, a, NULL, b); }
double vgo_relres_f64d(const vgo_geom* g, const double* a, const float* b) { return relres_impl(g, NULL, a, b); }

/* ------------------------------------------------------------- full step */

/* VortonSim::UpdateVortexParticleMethod with the shipped switches
 * (vortonSim.cpp:4117-4256): splat -vorticity, treecode boundary A,
 * cascade, Jacobian -> curl velocity grid, stretch/tilt, PSE, gather. */
void vgo_step_fields(const float* pos, float* vel, float* w, const float* size, size_t n, const vgo_geom* g, float dt,
                     float viscosity, int pse_mode, float* velgrid, float* vecpot, float* negvort) {
  const size_t cap = capacity(g);
  vgo_splat(pos, w, size, n, g, -1.0f, negvort);
  memset(vecpot, 0, cap * 3 * sizeof(float));
  vgo_boundary_vecpot(pos, w, size, n, g, 1, 1, vecpot);
  vgo_cascade(g, vecpot, negvort, 16);
  float* jac = (float*)malloc(cap * 9 * sizeof(float));
  vgo_jacobian(g, vecpot, jac);
  vgo_curl_from_jacobian(cap, jac, velgrid);
  vgo_jacobian(g, velgrid, jac);
  vgo_stretch(pos, w, n, g, jac, dt);
  free(jac);
  if (pse_mode == 0)
    vgo_pse_sequential(pos, w, size, n, g, viscosity, dt);
  else
    vgo_pse_symmetric(pos, w, size, n, g, viscosity, dt);
  vgo_gather(g, velgrid, pos, n, vel);
}

/* ExchangeHeat (VortonFluid/vortonSim.cpp:3905-3933). */
static void exchange_heat(const float* pos, float* d, const float* size, unsigned h, unsigned t, float kappa,
                          float dt) {
  const float range = 4.0f * size[h];
  const float range2 = range * range;
  const float sx = pos[3 * h] - pos[3 * t], sy = pos[3 * h + 1] - pos[3 * t + 1], sz = pos[3 * h + 2] - pos[3 * t + 2];
  const float dist2 = sx * sx + sy * sy + sz * sz;
  const float law = expf(-dist2 / range2);
  const float ratio = clampf_(2.0f * kappa * dt * law, -0.5f, 0.5f);
  const float ex = ratio * (d[h] - d[t]);
  d[h] -= ex;
  d[t] += ex;
}

/* DiffuseAndDissipateHeatPSESlice (VortonFluid/vortonSim.cpp:3954-4068), PHASE_BOTH over all cells. */
void vgo_heat_pse_sequential(const float* pos, float* d, const float* size, size_t n, const vgo_geom* g,
                             float kappa, float ambient, float dt) {
  cells_t c;
  cells_build(&c, pos, n, g);
  const float gain = clampf_(kappa * dt, -0.5f, 0.5f);
  const size_t nx = g->np[0], ny = g->np[1], nz = g->np[2], nxy = nx * ny;
  const size_t fo[3] = {1, nx, nxy};
  for (size_t z = 0; z + 1 < nz; ++z)
    for (size_t y = 0; y + 1 < ny; ++y)
      for (size_t x = 0; x + 1 < nx; ++x) {
        const size_t cell = x + y * nx + z * nxy;
        for (unsigned ih = 0; ih < c.count[cell]; ++ih) {
          const unsigned h = c.items[c.start[cell] + ih];
          for (unsigned it = ih + 1; it < c.count[cell]; ++it)
            exchange_heat(pos, d, size, h, c.items[c.start[cell] + it], kappa, dt);
          for (int k = 0; k < 3; ++k) {
            const size_t nb = cell + fo[k];
            for (unsigned it = 0; it < c.count[nb]; ++it)
              exchange_heat(pos, d, size, h, c.items[c.start[nb] + it], kappa, dt);
          }
          d[h] += gain * (ambient - d[h]);
        }
      }
  cells_free(&c);
}

/* Order-independent form: every pair the reference visits (same cell, or a
 * face neighbour along +x, +y or +z of a "here" cell strictly inside the point
 * range) exchanges with the densities from before the step, then every vorton
 * of a "here" cell relaxes toward ambient.  Differs from the reference's
 * in-place order by O((2 kappa dt)^2) of the density differences. */
void vgo_heat_pse_symmetric(const float* pos, float* d, const float* size, size_t n, const vgo_geom* g, float kappa,
                            float ambient, float dt) {
  cells_t c;
  cells_build(&c, pos, n, g);
  float* d0 = (float*)malloc((n ? n : 1) * sizeof(float));
  memcpy(d0, d, n * sizeof(float));
  const float gain = clampf_(kappa * dt, -0.5f, 0.5f);
  const int nx = (int)g->np[0], ny = (int)g->np[1], nz = (int)g->np[2];
  for (size_t i = 0; i < n; ++i) {
    unsigned id[3];
    vgo_indices_of_position(g, pos + 3 * i, id);
    const int ci[3] = {(int)id[0], (int)id[1], (int)id[2]};
    const int here_ok = ci[0] < nx - 1 && ci[1] < ny - 1 && ci[2] < nz - 1;
    double acc = 0.0;
    for (int s = -1; s <= 1; s += 2)
      for (int k = 0; k < 4; ++k) {
        if (k == 0 && s == 1) continue; /* same cell handled with s == -1 */
        const int dd[3] = {k == 1 ? s : 0, k == 2 ? s : 0, k == 3 ? s : 0};
        const int nc[3] = {ci[0] + dd[0], ci[1] + dd[1], ci[2] + dd[2]};
        if (nc[0] < 0 || nc[1] < 0 || nc[2] < 0 || nc[0] >= nx || nc[1] >= ny || nc[2] >= nz) continue;
        const int* lower = (s == 1) ? ci : nc;
        if (!(lower[0] < nx - 1 && lower[1] < ny - 1 && lower[2] < nz - 1)) continue;
        const size_t cell = (size_t)nc[0] + (size_t)nx * ((size_t)nc[1] + (size_t)ny * nc[2]);
        for (unsigned it = 0; it < c.count[cell]; ++it) {
          const unsigned j = c.items[c.start[cell] + it];
          if (j == i) continue;
          const unsigned here = (k == 0) ? (i < j ? (unsigned)i : j) : (s == 1 ? (unsigned)i : j);
          const float range = 4.0f * size[here];
          const float sx = pos[3 * i] - pos[3 * j], sy = pos[3 * i + 1] - pos[3 * j + 1],
                      sz = pos[3 * i + 2] - pos[3 * j + 2];
          const float law = expf(-(sx * sx + sy * sy + sz * sz) / (range * range));
          const float ratio = clampf_(2.0f * kappa * dt * law, -0.5f, 0.5f);
          acc += (double)ratio * ((double)d0[j] - (double)d0[i]);
        }
      }
    float v = (float)((double)d0[i] + acc);
    if (here_ok) v += gain * (ambient - v);
    d[i] = v;
  }
  free(d0);
  cells_free(&c);
}

/* PclOpKillAge::Operate (Particles/Operation/pclOpKillAge.cpp:22-47) with
 * Particles::Kill (Particles/particle.h:490-495): walk the slots; a slot whose
 * particle is too old takes the last particle and is tested again. */
void vgo_kill_age(const int* birth, size_t n, unsigned frame, int age_max, unsigned* order, size_t* m) {
  size_t size = n;
  for (size_t i = 0; i < n; ++i) order[i] = (unsigned)i;
  for (size_t i = 0; i < size;) {
    const int age = (int)(frame - (unsigned)birth[order[i]]);
    if (age > age_max) {
      order[i] = order[size - 1];
      --size;
    } else {
      ++i;
    }
  }
  *m = size;
}

/* PclOpWind::Operate (Particles/Operation/pclOpWind.cpp:18-42). */
void vgo_wind(float* vel, size_t n, const float wind[3], float wind_weight, float src_weight) {
  if (wind_weight == 0.0f && src_weight == 1.0f) return;
  const float term[3] = {wind_weight * wind[0], wind_weight * wind[1], wind_weight * wind[2]};
  for (size_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) vel[3 * i + c] = term[c] + src_weight * vel[3 * i + c];
}

/* ---------------------------------------------- density, baroclinic, surface */

/* UniformGrid<float>::Accumulate (uniformGrid.h:1278-1342): item spread over
 * the 8 corners of the containing cell with clamped trilinear weights, each
 * weight formed as ((wx * wy) * wz) * item. */
static void accumulate1(const vgo_geom* g, float* grid, const float p[3], float item) {
  unsigned idx[3];
  vgo_indices_of_position(g, p, idx);
  float tw[3], om[3];
  for (int a = 0; a < 3; ++a) {
    const float cmin = g->mn[a] + (float)idx[a] * g->cell[a];
    const float diff = p[a] - cmin;
    tw[a] = clampf_(diff * g->cpe[a], 0.0f, 1.0f);
    om[a] = 1.0f - tw[a];
  }
  const size_t nx = g->np[0], nxy = (size_t)g->np[0] * g->np[1];
  const size_t o = idx[0] + nx * (idx[1] + (size_t)g->np[1] * idx[2]);
  grid[o] += om[0] * om[1] * om[2] * item;
  grid[o + 1] += tw[0] * om[1] * om[2] * item;
  grid[o + nx] += om[0] * tw[1] * om[2] * item;
  grid[o + nx + 1] += tw[0] * tw[1] * om[2] * item;
  grid[o + nxy] += om[0] * om[1] * tw[2] * item;
  grid[o + nxy + 1] += tw[0] * om[1] * tw[2] * item;
  grid[o + nxy + nx] += om[0] * tw[1] * tw[2] * item;
  grid[o + nxy + nx + 1] += tw[0] * tw[1] * tw[2] * item;
}

/* VortonSim::PopulateDensityAndMassFractionGrids, density part
 * (VortonFluid/vortonSim.cpp:2911-3016): each particle's density times
 * (particle volume / cell volume), the particle volume taken from the first
 * particle (pi/6 size^3, Particles/particle.h:225-228), accumulated in
 * particle order together with a contribution grid of unit items; then
 * every point gains the ambient density times max(1 - contribution x
 * volume ratio, 0). */
void vgo_density_grid(const float* pos, const float* size, const float* density, size_t n, const vgo_geom* g,
                      float ambient, float* out) {
  const size_t pts = capacity(g);
  float* contrib = (float*)calloc(pts, sizeof(float));
  memset(out, 0, pts * sizeof(float));
  if (n > 0) {
    const float one_over_cell_volume = 1.0f / (g->cell[0] * g->cell[1] * g->cell[2]);
    const float pi_over_6 = PI_F / 6.0f;
    const float vorton_volume = pi_over_6 * size[0] * size[0] * size[0];
    const float volume_ratio = vorton_volume * one_over_cell_volume;
    for (size_t i = 0; i < n; ++i) {
      accumulate1(g, out, pos + 3 * i, density[i] * volume_ratio);
      accumulate1(g, contrib, pos + 3 * i, 1.0f);
    }
    for (size_t o = 0; o < pts; ++o) {
      const float pcls = contrib[o] * volume_ratio;
      const float clamped = minf_(pcls, 1.0f);
      out[o] += (1.0f - clamped) * ambient;
    }
  } else {
    for (size_t o = 0; o < pts; ++o) out[o] += 1.0f * ambient;
  }
  free(contrib);
}

/* ComputeGradient (Core/SpatialPartition/uniformGridMath.cpp:468-503,
 * 650-800): centred differences times half the reciprocal spacing inside,
 * one-sided differences times the reciprocal spacing on each face. */
void vgo_gradient(const vgo_geom* g, const float* v, float* grad3) {
  const float rs[3] = {1.0f / g->cell[0], 1.0f / g->cell[1], g->cell[2] > FLT_EPSILON ? 1.0f / g->cell[2] : 0.0f};
  const float hrs[3] = {0.5f * rs[0], 0.5f * rs[1], 0.5f * rs[2]};
  const size_t nx = g->np[0], ny = g->np[1], nz = g->np[2];
  const size_t st[3] = {1, nx, nx * ny};
  for (size_t z = 0; z < nz; ++z)
    for (size_t y = 0; y < ny; ++y)
      for (size_t x = 0; x < nx; ++x) {
        const size_t o = x + nx * (y + ny * z);
        const size_t id[3] = {x, y, z};
        const size_t last[3] = {nx - 1, ny - 1, nz - 1};
        for (int a = 0; a < 3; ++a) {
          float d;
          if (id[a] == 0)
            d = (v[o + st[a]] - v[o]) * rs[a];
          else if (id[a] == last[a])
            d = (v[o] - v[o - st[a]]) * rs[a];
          else
            d = (v[o + st[a]] - v[o - st[a]]) * hrs[a];
          grad3[3 * o + a] = d;
        }
      }
}

/* Baroclinic generation on the density-grid path of
 * VortonSim::GenerateBaroclinicVorticity (vortonSim.cpp:3407-3547) with
 * GenerateBaroclinicVorticitySlice (vortonSim.cpp:3318-3392): density grid,
 * its gradient, the gradient interpolated at each vorton, then
 * angvel += (0.5 * (grad x (g * (1 / ambient)))) * dt where the gradient is
 * finite.  Returns 0 (and changes nothing) when the grid has no extent along
 * gravity (|g . extent| < FLT_EPSILON, vortonSim.cpp:3417-3421). */
int vgo_baroclinic(const float* pos, float* angvel, const float* size, const float* density, size_t n,
                   const vgo_geom* g, const float grav[3], float ambient, float dt) {
  const float gdot = grav[0] * g->ext[0] + grav[1] * g->ext[1] + grav[2] * g->ext[2];
  if (fabsf(gdot) < FLT_EPSILON) return 0;
  const size_t pts = capacity(g);
  float* dens = (float*)malloc(pts * sizeof(float));
  float* grad = (float*)malloc(pts * 3 * sizeof(float));
  vgo_density_grid(pos, size, density, n, g, ambient, dens);
  vgo_gradient(g, dens, grad);
  const float one_over_density = 1.0f / ambient;
  const float pg[3] = {grav[0] * one_over_density, grav[1] * one_over_density, grav[2] * one_over_density};
  for (size_t i = 0; i < n; ++i) {
    float d[3];
    vgo_interpolate3(g, grad, pos + 3 * i, d);
    if (!(isfinite(d[0]) && isfinite(d[1]) && isfinite(d[2]))) continue;
    const float b[3] = {d[1] * pg[2] - d[2] * pg[1], d[2] * pg[0] - d[0] * pg[2], d[0] * pg[1] - d[1] * pg[0]};
    for (int a = 0; a < 3; ++a) angvel[3 * i + a] = angvel[3 * i + a] + 0.5f * b[a] * dt;
  }
  free(dens);
  free(grad);
  return 1;
}

/* FindValueStats (uniformGridMath.cpp:554-590): min, max and the mean and
 * standard deviation from float sums in point order. */
static void value_stats(const float* v, size_t n, float* mn, float* mx, float* mean, float* sd) {
  float lo = FLT_MAX, hi = -FLT_MAX, sum = 0.0f, sum2 = 0.0f;
  for (size_t i = 0; i < n; ++i) {
    lo = minf_(v[i], lo);
    hi = maxf_(v[i], hi);
    sum += v[i];
    sum2 += v[i] * v[i];
  }
  *mn = lo;
  *mx = hi;
  *mean = sum / (float)n;
  const float mean2 = sum2 / (float)n;
  const float variance = mean2 - *mean * *mean;
  *sd = sqrtf(maxf_(variance, 0.0f));
}

static void update_sdf(float* here, float cand) {
  if (fabsf(cand) < fabsf(*here)) *here = cand;
}

/* PopulateSignedDistanceGridFromDensityGrid (vortonSim.cpp:3266-3290) with
 * ComputeImmediateSDFFromDensity_Nearest and
 * ComputeRemainingSDFFromImmediateSDF_Nearest (Particles/Operation/
 * pclOpEmit.cpp:696-881, 882-1060), serial form:
 *   1. density statistics; inside density = min(max, mean + stddev);
 *   2. every cell's +x, +y, +z edges from its min corner that cross the
 *      surface (density - ambient changes sign) pin both end points with the
 *      fraction of a spacing to the crossing (negative inside), keeping the
 *      value of least magnitude;
 *   3. two sweeps (all axes forward, then all backward) set each unpinned
 *      point from its backward neighbour of least |value| plus one spacing
 *      of that neighbour's sign, where that is closer;
 *   4. points still at FLT_MAX become NaN.
 * `sumstats` selects the statistics' summation: 0 float sums in point order
 * (the reference's), 1 double sums (a parallel reduction's reference). */
void vgo_signed_distance(const vgo_geom* g, const float* density, float ambient, int sumstats, float* sdf) {
  const size_t pts = capacity(g);
  float dmin, dmax, dmean, dsd;
  if (sumstats == 0) {
    value_stats(density, pts, &dmin, &dmax, &dmean, &dsd);
  } else {
    double s = 0.0, s2 = 0.0;
    dmin = FLT_MAX;
    dmax = -FLT_MAX;
    for (size_t i = 0; i < pts; ++i) {
      dmin = minf_(density[i], dmin);
      dmax = maxf_(density[i], dmax);
      s += density[i];
      s2 += (double)density[i] * density[i];
    }
    dmean = (float)(s / (double)pts);
    const float mean2 = (float)(s2 / (double)pts);
    const float variance = mean2 - dmean * dmean;
    dsd = sqrtf(maxf_(variance, 0.0f));
  }
  const float inside = minf_(dmax, dmean + dsd);
  const float denom = inside - ambient;
  const size_t nx = g->np[0], ny = g->np[1], nz = g->np[2], nxy = nx * ny;
  int* pinned = (int*)calloc(pts, sizeof(int));
  for (size_t i = 0; i < pts; ++i) sdf[i] = FLT_MAX;
  for (size_t z = 0; z + 1 < nz; ++z)
    for (size_t y = 0; y + 1 < ny; ++y)
      for (size_t x = 0; x + 1 < nx; ++x) {
        const size_t o = x + nx * (y + ny * z);
        const size_t nb[3] = {o + 1, o + nx, o + nxy};
        const float here = density[o] - ambient;
        for (int a = 0; a < 3; ++a) {
          const float other = density[nb[a]] - ambient;
          float ch, cn;
          if (here <= 0.0f && 0.0f < other) {
            const float t = minf_(other / denom, 1.0f);
            ch = (1.0f - t) * g->cell[a];
            cn = -t * g->cell[a];
          } else if (here > 0.0f && 0.0f >= other) {
            const float t = minf_(here / denom, 1.0f);
            ch = -t * g->cell[a];
            cn = (1.0f - t) * g->cell[a];
          } else {
            continue;
          }
          pinned[o] = 1;
          pinned[nb[a]] = 1;
          update_sdf(&sdf[o], ch);
          update_sdf(&sdf[nb[a]], cn);
        }
      }
  for (int pass = 0; pass < 2; ++pass) {
    const long inc = pass ? -1 : 1;
    const long b[3] = {pass ? (long)nx - 1 : 0, pass ? (long)ny - 1 : 0, pass ? (long)nz - 1 : 0};
    const long e[3] = {pass ? -1 : (long)nx, pass ? -1 : (long)ny, pass ? -1 : (long)nz};
    for (long z = b[2]; z != e[2]; z += inc)
      for (long y = b[1]; y != e[1]; y += inc)
        for (long x = b[0]; x != e[0]; x += inc) {
          const size_t o = (size_t)x + nx * ((size_t)y + ny * (size_t)z);
          if (pinned[o]) continue;
          const float sx = (x != b[0]) ? sdf[o - inc] : FLT_MAX;
          const float sy = (y != b[1]) ? sdf[o - inc * (long)nx] : FLT_MAX;
          const float sz = (z != b[2]) ? sdf[o - inc * (long)nxy] : FLT_MAX;
          const float ax = fabsf(sx), ay = fabsf(sy), az = fabsf(sz);
          float nbv, sp;
          if (ax <= ay) {
            if (ax <= az) {
              nbv = sx;
              sp = g->cell[0];
            } else {
              nbv = sz;
              sp = g->cell[2];
            }
          } else if (ay <= az) {
            nbv = sy;
            sp = g->cell[1];
          } else {
            nbv = sz;
            sp = g->cell[2];
          }
          update_sdf(&sdf[o], nbv + copysignf(sp, nbv));
        }
  }
  for (size_t i = 0; i < pts; ++i)
    if (sdf[i] == FLT_MAX) sdf[i] = NAN;
  free(pinned);
}

/* ------------------------------------------------------------ marching cubes */

/* Cell corners (x, y, z offsets) and edges (corner pairs in the order the
 * reference interpolates them), the layout of Render/Resource/
 * marchingCubes.cpp:590-622, 800-816.  The triangulation itself is generated
 * here, not taken from a table: on each cube face the crossing edges are
 * joined into segments (on a face with four crossings, each segment cuts off
 * one corner below the iso level), segments are oriented so that the
 * corners below the iso level lie on one fixed side, chained into loops, and
 * each loop is fanned from its first edge. */
static const int mc_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                    {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const int mc_edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                   {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
static const int mc_face[6][5] = {{0, 1, 2, 3, -3}, {4, 5, 6, 7, 3}, {0, 1, 5, 4, -2},
                                  {3, 2, 6, 7, 2},  {0, 3, 7, 4, -1}, {1, 2, 6, 5, 1}};  /* corners, then +-axis */

static int mc_edge_of(int a, int b) {
  for (int e = 0; e < 12; ++e)
    if ((mc_edge[e][0] == a && mc_edge[e][1] == b) || (mc_edge[e][0] == b && mc_edge[e][1] == a)) return e;
  return -1;
}

/* Orientation of segment a -> b on a face with outward normal axis `ax`
 * (+-1..3): the sign of ((B - A) x (P - A)) . n for the edge midpoints A, B and
 * a corner P below the iso level.  Coordinates are doubled so they stay integers. */
static int mc_side(int a, int b, int pin, int ax) {
  int A[3], B[3], P[3], u[3], v[3], cr[3];
  for (int k = 0; k < 3; ++k) {
    A[k] = mc_corner[mc_edge[a][0]][k] + mc_corner[mc_edge[a][1]][k];
    B[k] = mc_corner[mc_edge[b][0]][k] + mc_corner[mc_edge[b][1]][k];
    P[k] = 2 * mc_corner[pin][k];
    u[k] = B[k] - A[k];
    v[k] = P[k] - A[k];
  }
  cr[0] = u[1] * v[2] - u[2] * v[1];
  cr[1] = u[2] * v[0] - u[0] * v[2];
  cr[2] = u[0] * v[1] - u[1] * v[0];
  const int axis = (ax > 0 ? ax : -ax) - 1;
  return ax > 0 ? cr[axis] : -cr[axis];
}

/* Triangles of case `mask` (bit c set: corner c below the iso level) as edge
 * triples; returns their count. */
static int mc_case(int mask, int tri[15]) {
  int next[12];
  for (int e = 0; e < 12; ++e) next[e] = -1;
  for (int f = 0; f < 6; ++f) {
    const int* cc = mc_face[f];
    int ee[4], cr[4], nc = 0;
    for (int k = 0; k < 4; ++k) {
      ee[k] = mc_edge_of(cc[k], cc[(k + 1) % 4]);
      if (((mask >> cc[k]) & 1) != ((mask >> cc[(k + 1) % 4]) & 1)) cr[nc++] = k;
    }
    int seg[2][3], ns = 0;
    if (nc == 2) {
      int pin = -1;
      for (int k = 0; k < 4 && pin < 0; ++k)
        if ((mask >> cc[k]) & 1) pin = cc[k];
      seg[0][0] = ee[cr[0]];
      seg[0][1] = ee[cr[1]];
      seg[0][2] = pin;
      ns = 1;
    } else if (nc == 4) {
      for (int k = 0; k < 4; ++k)
        if ((mask >> cc[k]) & 1) {
          seg[ns][0] = ee[(k + 3) % 4];
          seg[ns][1] = ee[k];
          seg[ns][2] = cc[k];
          ++ns;
        }
    }
    for (int s = 0; s < ns; ++s) {
      const int a = seg[s][0], b = seg[s][1];
      if (mc_side(a, b, seg[s][2], cc[4]) < 0)
        next[a] = b;
      else
        next[b] = a;
    }
  }
  int seen[12] = {0}, nt = 0;
  for (int e = 0; e < 12; ++e) {
    if (next[e] < 0 || seen[e]) continue;
    int loop[12], n = 0, x = e;
    do {
      loop[n++] = x;
      seen[x] = 1;
      x = next[x];
    } while (x != e && n < 12);
    for (int i = 1; i + 1 < n; ++i) {
      tri[3 * nt] = loop[0];
      tri[3 * nt + 1] = loop[i];
      tri[3 * nt + 2] = loop[i + 1];
      ++nt;
    }
  }
  return nt;
}

/* VertexInterp (marchingCubes.cpp:228-250): the end point itself within 1e-5
 * (compared in double, as the double literal makes it), else the linear
 * crossing p1 + mu (p2 - p1). */
static void mc_interp(float iso, const float p1[3], const float p2[3], float v1, float v2, float out[3]) {
  if ((double)fabsf(iso - v1) < 0.00001) {
    memcpy(out, p1, 3 * sizeof(float));
    return;
  }
  if ((double)fabsf(iso - v2) < 0.00001) {
    memcpy(out, p2, 3 * sizeof(float));
    return;
  }
  if ((double)fabsf(v1 - v2) < 0.00001) {
    memcpy(out, p1, 3 * sizeof(float));
    return;
  }
  const float mu = (iso - v1) / (v2 - v1);
  for (int k = 0; k < 3; ++k) out[k] = p1[k] + mu * (p2[k] - p1[k]);
}

/* ExtractIsoLevel_Slice + PolygoniseCellWithNormal (marchingCubes.cpp:
 * 580-760, 762-866) on grid g of scalar values: cells in z, y, x order; for
 * each triangle the three vertex positions (9 floats) and its unit face
 * normal (p1 - p0) x (p2 - p0) / sqrt(|.|^2 + FLT_MIN) repeated for the three
 * vertices (9 floats).  Corner positions are min + index x spacing.  Writes
 * at most cap triangles; returns how many the grid makes. */
size_t vgo_marching_cubes(const vgo_geom* g, const float* v, float iso, float* verts, float* normals, size_t cap) {
  static int table_ready = 0;
  static int cnt[256], tri[256][15];
  if (!table_ready) {
    for (int m = 0; m < 256; ++m) cnt[m] = mc_case(m, tri[m]);
    table_ready = 1;
  }
  const size_t nx = g->np[0], ny = g->np[1], nz = g->np[2], nxy = nx * ny;
  size_t out = 0;
  for (size_t z = 0; z + 1 < nz; ++z)
    for (size_t y = 0; y + 1 < ny; ++y)
      for (size_t x = 0; x + 1 < nx; ++x) {
        const size_t o = x + nx * (y + ny * z);
        float val[8], p[8][3];
        int mask = 0;
        const float gp[3] = {(float)x * g->cell[0] + g->mn[0], (float)y * g->cell[1] + g->mn[1],
                             (float)z * g->cell[2] + g->mn[2]};
        const float hi[3] = {gp[0] + g->cell[0], gp[1] + g->cell[1], gp[2] + g->cell[2]};
        for (int c = 0; c < 8; ++c) {
          const int* d = mc_corner[c];
          val[c] = v[o + d[0] + nx * d[1] + nxy * d[2]];
          for (int k = 0; k < 3; ++k) p[c][k] = d[k] ? hi[k] : gp[k];
          if (val[c] < iso) mask |= 1 << c;
        }
        if (cnt[mask] == 0) continue;
        float vl[12][3];
        for (int e = 0; e < 12; ++e) {
          const int a = mc_edge[e][0], b = mc_edge[e][1];
          if (((mask >> a) & 1) != ((mask >> b) & 1)) mc_interp(iso, p[a], p[b], val[a], val[b], vl[e]);
        }
        for (int t = 0; t < cnt[mask]; ++t, ++out) {
          if (out >= cap) continue;
          const float* q0 = vl[tri[mask][3 * t]];
          const float* q1 = vl[tri[mask][3 * t + 1]];
          const float* q2 = vl[tri[mask][3 * t + 2]];
          float* dst = verts + 9 * out;
          memcpy(dst, q0, 12);
          memcpy(dst + 3, q1, 12);
          memcpy(dst + 6, q2, 12);
          if (normals) {
            const float u[3] = {q1[0] - q0[0], q1[1] - q0[1], q1[2] - q0[2]};
            const float w[3] = {q2[0] - q0[0], q2[1] - q0[1], q2[2] - q0[2]};
            const float n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
            const float r = 1.0f / sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2] + FLT_MIN);
            for (int k = 0; k < 3; ++k) {
              normals[9 * out + 3 * k] = n[0] * r;
              normals[9 * out + 3 * k + 1] = n[1] * r;
              normals[9 * out + 3 * k + 2] = n[2] * r;
            }
          }
        }
      }
  return out;
}

/* The generated triangulation: count[256] and up to 5 edge triples per case. */
void vgo_marching_cubes_table(int* count, int* tri15) {
  for (int m = 0; m < 256; ++m) count[m] = mc_case(m, tri15 + 15 * m);
}

/* ------------------------------------------------- fluid-body boundary conditions */

typedef struct {
  float x, y, z;
} v3_t;
static v3_t v3(float x, float y, float z) {
  v3_t r = {x, y, z};
  return r;
}
static v3_t v3add(v3_t a, v3_t b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3_t v3sub(v3_t a, v3_t b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3_t v3mul(v3_t a, float f) { return v3(a.x * f, a.y * f, a.z * f); }
static float v3dot(v3_t a, v3_t b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3_t v3cross(v3_t a, v3_t b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static float v3mag(v3_t a) { return sqrtf(v3dot(a, a)); }
/* Vec3::GetDirFast (vec3.h:429) and GetDir (vec3.h:428). */
static v3_t v3dirfast(v3_t a) { return v3mul(a, vgo_finvsqrtf(v3dot(a, a) + FLT_MIN)); }
static v3_t v3dir(v3_t a) { return v3mul(v3mul(a, 1.0f), 1.0f / sqrtf(v3dot(a, a) + FLT_MIN)); }

/* A rigid body of the fluid-body simulation, 32 floats: [0] shape (0 sphere,
 * 1 box), [1] hole (box only), [2..4] position, [5..7] velocity, [8..10]
 * angular velocity, [11..19] orientation rows, [20..22] sphere radius (x) or
 * box dimensions, [23] temperature, [24] thermal conductivity. */
typedef struct {
  int box;
  float parity, brad;
  v3_t pos, vel, angvel, row[3];
  v3_t pn[6];
  float pw[6];
  float temperature, conductivity;
} body_t;

/* PhysicalObject with SphereShape, or ConvexPolytope made by
 * ConvexPolytope_MakeBox (Collision/convexPolytope.cpp:346-376). */
static body_t body_load(const float* q) {
  body_t b;
  memset(&b, 0, sizeof(b));
  b.box = q[0] != 0.0f;
  b.parity = (b.box && q[1] != 0.0f) ? -1.0f : 1.0f;
  b.pos = v3(q[2], q[3], q[4]);
  b.vel = v3(q[5], q[6], q[7]);
  b.angvel = v3(q[8], q[9], q[10]);
  for (int r = 0; r < 3; ++r) b.row[r] = v3(q[11 + 3 * r], q[12 + 3 * r], q[13 + 3 * r]);
  b.temperature = q[23];
  b.conductivity = q[24];
  if (!b.box) {
    b.brad = q[20];
  } else {
    const float x = q[20] * 0.5f, y = q[21] * 0.5f, z = q[22] * 0.5f;
    const float half[3] = {x, y, z};
    for (int a = 0; a < 3; ++a) {
      float n1[3] = {0, 0, 0}, n2[3] = {0, 0, 0};
      n1[a] = 1.0f;
      n2[a] = -1.0f;
      b.pn[2 * a] = v3(n1[0], n1[1], n1[2]);
      b.pn[2 * a + 1] = v3(n2[0], n2[1], n2[2]);
      b.pw[2 * a] = b.pw[2 * a + 1] = half[a];
    }
    if (b.parity < 0.0f) {
      const float thin = 1.0f - FLT_EPSILON;
      b.brad = thin * minf_(minf_(x, y), z);
    } else {
      const float fatten = 1.0f + FLT_EPSILON;
      b.brad = 0.5f * fatten * v3mag(v3(q[20], q[21], q[22]));
    }
  }
  return b;
}

/* Mat33::TransformByTranspose (mat33.h:131-134) and Transform (mat33.h:108-113). */
static v3_t xform_t(const body_t* b, v3_t v) { return v3(v3dot(b->row[0], v), v3dot(b->row[1], v), v3dot(b->row[2], v)); }
static v3_t xform(const body_t* b, v3_t v) {
  return v3(v3dot(v3(b->row[0].x, b->row[1].x, b->row[2].x), v), v3dot(v3(b->row[0].y, b->row[1].y, b->row[2].y), v),
            v3dot(v3(b->row[0].z, b->row[1].z, b->row[2].z), v));
}

/* ConvexPolytope::ContactDistance (convexPolytope.cpp:97-144): the largest
 * plane distance of the point in body space, times the parity. */
static float contact_distance(const body_t* b, v3_t q, int* idx) {
  const v3_t r = xform_t(b, v3sub(q, b->pos));
  float largest = -FLT_MAX;
  for (int i = 0; i < 6; ++i) {
    const float d = v3dot(r, b->pn[i]) - b->pw[i];
    if (d > largest) {
      largest = d;
      *idx = i;
    }
  }
  return largest * b->parity;
}

/* ConvexPolytope::CollisionDistance with velocities (convexPolytope.cpp:151-196). */
static float collision_distance(const body_t* b, v3_t q, v3_t qv, int* idx) {
  const v3_t r = xform_t(b, v3sub(q, b->pos));
  const v3_t rv = xform_t(b, v3sub(qv, b->vel));
  float largest = -FLT_MAX;
  for (int i = 0; i < 6; ++i) {
    const float d = v3dot(r, b->pn[i]) - b->pw[i];
    if (d > largest) {
      const float speed = v3dot(rv, b->pn[i]) * b->parity;
      if (speed <= 0.0f || d >= 0.0f || b->parity < 0.0f) {
        largest = d;
        *idx = i;
      }
    }
  }
  return largest * b->parity;
}

/* ConvexPolytope::ContactPoint (convexPolytope.cpp:325-339). */
static v3_t contact_point(const body_t* b, v3_t q, int idx, float dist, v3_t* n) {
  *n = v3mul(xform(b, b->pn[idx]), b->parity);
  return v3sub(q, v3mul(*n, dist));
}

/* Vorton::AccumulateVelocity (vorton.h:240-243): the reference velocity law
 * of one vorton at a query point, spreading factors 1. */
static v3_t vorton_velocity(v3_t q, v3_t p, v3_t w, float size) {
  float acc[3] = {0.0f, 0.0f, 0.0f};
  const float qq[3] = {q.x, q.y, q.z}, pp[3] = {p.x, p.y, p.z}, ww[3] = {w.x, w.y, w.z};
  accum(0, acc, qq, pp, ww, size, 1.0f, 1.0f);
  return v3(acc[0], acc[1], acc[2]);
}

/* FluidBodySim::CollideVortonsSlice (FluidBodySim/fluidBodySim.cpp:759-1180)
 * with the shipped switches (no-slip / no-through boundary respecting the
 * ambient flow without the vorton's own old contribution, the vorton placed
 * outside the body and bounced, vorticity by the Brinkman penalty blended with
 * gain 0.1 and the body's spin, heat conducted, smoothed-particle form so no
 * linear impulse), for each body in turn over all particles.  Per body out9
 * receives linear impulse, angular impulse, heat to body, sum of particle
 * temperatures and the collision count. */
void vgo_collide_vortons(float* pos, float* vel, float* angvel, const float* size, float* density, size_t n,
                         const float* bodies, int nb, float ambient, float specific_heat, float* out9) {
  const float thin = 1.0f - FLT_EPSILON, fatten = 1.0f + FLT_EPSILON, nudge = 1.0f + 1.0e-4f;
  const float impact = 1.0f + 0.01f;
  for (int k = 0; k < nb; ++k) {
    const body_t B = body_load(bodies + 32 * k);
    v3_t ang_imp = v3(0.0f, 0.0f, 0.0f);
    float heat = 0.0f, sum_t = 0.0f;
    size_t count = 0;
    const float one_over_cp = 1.0f / specific_heat;
    size_t incr = 1, repeat = 0;
    for (size_t i = 0; i < n; i += incr) {
      repeat = (0 == incr) ? repeat + 1 : 0;
      incr = 1;
      v3_t p = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      v3_t v = v3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
      v3_t w = v3(angvel[3 * i], angvel[3 * i + 1], angvel[3 * i + 2]);
      const float r = size[i] * 0.5f, r2 = r * r;
      const v3_t s2v = v3sub(p, B.pos);
      const float fs2v = v3mag(s2v);
      const float bnd = 1.5f * r;
      int broad;
      if (B.parity < 0.0f)
        broad = fs2v > maxf_(B.brad - bnd, 0.0f) * thin;
      else
        broad = fs2v < (B.brad + bnd) * fatten;
      if (!broad) continue;
      v3_t cw, n3;
      float cdist;
      if (!B.box) {
        const v3_t dir = v3mul(s2v, 1.0f / fs2v);
        const v3_t crel = v3mul(dir, B.brad);
        cw = v3add(crel, B.pos);
        n3 = dir;
        cdist = fs2v - B.brad;
      } else {
        int idx = 0;
        cdist = contact_distance(&B, p, &idx);
        if (!(cdist < bnd)) continue;
        cw = contact_point(&B, p, idx, cdist, &n3);
        if (B.parity < 0.0f && repeat < 5 && cdist < r) incr = 0;
      }
      ++count;
      const v3_t vbody = B.vel;
      v3_t vort_old = v3mul(w, 2.0f);
      const v3_t due_old = vorton_velocity(cw, p, w, size[i]);
      const v3_t flow = v3sub(v3sub(v, due_old), vbody);
      (void)v3dirfast(flow);
      const float disp = cdist < r ? r : cdist;
      p = v3add(cw, v3mul(v3mul(n3, disp), nudge));
      {
        const v3_t vrel = v3sub(v, vbody);
        const float speed_n = v3dot(vrel, n3);
        const v3_t impulse = v3mul(n3, -speed_n);
        v = v3add(v, v3mul(impulse, impact));
      }
      if (repeat >= 1) {
        v = v3(0.0f, 0.0f, 0.0f);
        w = v3(0.0f, 0.0f, 0.0f);
        vort_old = w;
      } else {
        /* Vorton::AssignVorticityByPenalty (vorton.h:275-306) */
        const v3_t rel = v3sub(cw, p);
        const v3_t vd = v3sub(v, vbody);
        const float dist = v3mag(rel) - size[i] * 0.4f;
        const v3_t vdir = v3dir(v3cross(vd, rel));
        const float vmag = v3mag(vd) / dist;
        w = v3mul(v3mul(vdir, vmag), 0.5f);
      }
      w = v3add(w, v3sub(v3mul(B.angvel, 1.0f), v3mul(vort_old, 0.5f)));
      {
        const float gain = 0.1f, one_minus = 1.0f - gain;
        w = v3mul(v3add(v3mul(v3mul(w, 2.0f), gain), v3mul(vort_old, one_minus)), 0.5f);
      }
      const v3_t angdiff = v3mul(v3sub(vort_old, v3mul(w, 2.0f)), 0.5f);
      {
        const float t_old = 300.0f * ambient / density[i];
        const float t_diff = B.temperature - t_old;
        const float t_gain = clampf_(B.conductivity * r * 0.03f * specific_heat, -0.5f, 0.5f);
        const float t_change = t_diff * t_gain;
        const float heat_ex = t_change * one_over_cp;
        const float t_new = t_old + t_change;
        density[i] = ambient * 300.0f / t_new;
        heat -= heat_ex;
        sum_t += t_old;
      }
      {
        const float pi_over_6 = PI_F / 6.0f;
        const float mass = density[i] * (pi_over_6 * size[i] * size[i] * size[i]);
        const float moi = 0.4f * mass * r2;
        ang_imp = v3add(ang_imp, v3mul(angdiff, moi));
      }
      pos[3 * i] = p.x, pos[3 * i + 1] = p.y, pos[3 * i + 2] = p.z;
      vel[3 * i] = v.x, vel[3 * i + 1] = v.y, vel[3 * i + 2] = v.z;
      angvel[3 * i] = w.x, angvel[3 * i + 1] = w.y, angvel[3 * i + 2] = w.z;
    }
    float* o = out9 + 9 * k;
    o[0] = o[1] = o[2] = 0.0f;
    o[3] = ang_imp.x, o[4] = ang_imp.y, o[5] = ang_imp.z;
    o[6] = heat, o[7] = sum_t, o[8] = (float)count;
  }
}

/* FluidBodySim::CollideTracersSlice (fluidBodySim.cpp:1300-1455) for each
 * body in turn: a tracer in contact is placed outside the body (sphere: at
 * bounding radius plus its radius along its direction from the centre; box:
 * from the contact point along the face normal) and its velocity bounced
 * with impact coefficient 1.01; per body out6 receives the linear and angular
 * impulses on the body (tracer mass = density x volume). */
void vgo_collide_tracers(float* pos, float* vel, const float* size, const float* density, size_t n,
                         const float* bodies, int nb, float* out6) {
  const float thin = 1.0f - FLT_EPSILON, fatten = 1.0f + FLT_EPSILON, nudge = 1.0f + 1.0e-4f;
  const float impact = 1.0f + 0.01f;
  for (int k = 0; k < nb; ++k) {
    const body_t B = body_load(bodies + 32 * k);
    v3_t lin = v3(0.0f, 0.0f, 0.0f), ang = v3(0.0f, 0.0f, 0.0f);
    size_t incr = 1, repeat = 0;
    for (size_t i = 0; i < n; i += incr) {
      repeat = (0 == incr) ? repeat + 1 : 0;
      incr = 1;
      v3_t p = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      v3_t v = v3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
      const float r = size[i] * 0.5f;
      const v3_t s2t = v3sub(p, B.pos);
      const float fs2t = v3mag(s2t);
      int broad;
      if (B.parity < 0.0f)
        broad = fs2t > maxf_(B.brad - r, 0.0f) * thin;
      else
        broad = fs2t < (B.brad + r) * fatten;
      if (!broad) continue;
      v3_t cp, n3, disp_new;
      if (!B.box) {
        const float rescale = (B.brad + r) * (1.0f + FLT_EPSILON) / fs2t;
        disp_new = v3mul(s2t, rescale);
        cp = disp_new;
        n3 = v3dirfast(s2t);
      } else {
        int idx = 0;
        const float cdist = collision_distance(&B, p, v, &idx);
        if (!(cdist < r)) continue;
        cp = contact_point(&B, p, idx, cdist, &n3);
        disp_new = v3sub(v3add(cp, v3mul(v3mul(n3, r), nudge)), B.pos);
        if (B.parity < 0.0f && repeat < 5) incr = 0;
      }
      const v3_t vrot = v3cross(B.angvel, disp_new);
      const v3_t vbody = v3add(B.vel, vrot);
      const v3_t vrel = v3sub(v, vbody);
      const float speed_n = v3dot(vrel, n3);
      const v3_t impulse = v3mul(n3, -speed_n);
      const v3_t vnew = v3add(v, v3mul(impulse, impact));
      const float pi_over_6 = PI_F / 6.0f;
      const float mass = density[i] * (pi_over_6 * size[i] * size[i] * size[i]);
      const v3_t li = v3mul(v3sub(v, vnew), mass);
      lin = v3add(lin, li);
      ang = v3add(ang, v3cross(v3sub(cp, B.pos), li));
      p = v3add(B.pos, disp_new);
      pos[3 * i] = p.x, pos[3 * i + 1] = p.y, pos[3 * i + 2] = p.z;
      vel[3 * i] = vnew.x, vel[3 * i + 1] = vnew.y, vel[3 * i + 2] = vnew.z;
    }
    float* o = out6 + 6 * k;
    o[0] = lin.x, o[1] = lin.y, o[2] = lin.z, o[3] = ang.x, o[4] = ang.y, o[5] = ang.z;
  }
}

/* FluidBodySim::RemoveEmbeddedParticles (fluidBodySim.cpp:365-417): for each
 * body in turn, particles within its bounding sphere that lie inside it
 * (sphere: inside the bounding sphere; box: contact distance below the
 * particle's radius) are removed by moving the last particle into their slot
 * (Particles::Kill) and testing the slot again.  order receives the
 * survivors' original indices in the order left. */
void vgo_remove_embedded(const float* pos, const float* size, size_t n, const float* bodies, int nb, unsigned* order,
                         size_t* m) {
  size_t cnt = n;
  for (size_t i = 0; i < n; ++i) order[i] = (unsigned)i;
  for (int k = 0; k < nb; ++k) {
    const body_t B = body_load(bodies + 32 * k);
    for (size_t i = 0; i < cnt;) {
      const unsigned j = order[i];
      const v3_t p = v3(pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]);
      const float d = v3mag(v3sub(p, B.pos));
      int kill = 0;
      if (d < B.brad) {
        if (!B.box) {
          kill = 1;
        } else {
          int idx = 0;
          kill = contact_distance(&B, p, &idx) < size[j] * 0.5f;
        }
      }
      if (kill) {
        order[i] = order[cnt - 1];
        --cnt;
      } else {
        ++i;
      }
    }
  }
  *m = cnt;
}

/* ------------------------------------------------------------------ emitters */

/* The counter-based jitter stream of the device emitter (used in place of
 * the C library's rand() when asked): draw d of stream `seed` is the
 * MurmurHash3 32-bit finalizer (fmix32, Austin Appleby, public domain) of the
 * low word of d keyed by the seed and the high word, scaled to
 * [0, RAND_MAX]. */
static uint32_t fmix32_(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

int vgo_jitter_hash(unsigned seed, uint64_t d) {
  const uint32_t key = fmix32_(seed ^ ((uint32_t)(d >> 32) * 0x9e3779b9u + 0x7f4a7c15u));
  const uint32_t h = fmix32_((uint32_t)d ^ key);
  return (int)(((uint64_t)h * ((uint64_t)RAND_MAX + 1u)) >> 32);
}

int vgo_rand_max(void) { return RAND_MAX; }

/* The next jitter draw: the C library's rand() (the reference's source) or
 * the hash stream. */
static int draw_(int host_rand, unsigned seed, uint64_t* d) {
  const uint64_t k = (*d)++;
  return host_rand ? rand() : vgo_jitter_hash(seed, k);
}

/* RandomSpread (Core/Math/math.h:183-188): spread * (r / RAND_MAX - 1/2). */
static float spread_(float spread, int r) {
  const float one_over_rand_max = 1.0f / (float)RAND_MAX;
  return spread * ((float)r * one_over_rand_max - 0.5f);
}

/* RandomSpread of a Vec3 (Core/Math/vec3.h:540-545): the three calls are
 * arguments of one constructor, which the compilers the reference targets
 * evaluate last to first, so z draws first. */
static void spread3_(const float s[3], int host_rand, unsigned seed, uint64_t* d, float out[3]) {
  out[2] = spread_(s[2], draw_(host_rand, seed, d));
  out[1] = spread_(s[1], draw_(host_rand, seed, d));
  out[0] = spread_(s[0], draw_(host_rand, seed, d));
}

/* PclOpEmit::Emit (Particles/Operation/pclOpEmit.cpp:77-186): multiplier^3
 * particles per cell of g, cells in z, y, x order and sub-cells likewise, at
 * min corner + (it / m) spacing + half a sub-cell + a jitter below half a
 * sub-cell.  With vortons, each vorton's density deviation from the ambient
 * 1 is accumulated onto g (PopulateDensityDeviationGridFromParticles,
 * pclOpEmit.cpp:29-57); nothing is emitted (and nothing drawn) when the
 * deviation is zero everywhere, else a particle is kept where the
 * interpolated deviation is at least half the largest magnitude, with
 * density deviation + that magnitude.  Outputs: position, density, size of
 * each particle kept, up to max; *count all kept. */
void vgo_emit_grid(const vgo_geom* g, unsigned m, const float* vpos, const float* vdens, size_t nv, int use_vortons,
                   int host_rand, unsigned seed, float* pos_out, float* dens_out, float* size_out, size_t max,
                   size_t* count) {
  const float ambient = 1.0f;
  const float* sp = g->cell;
  const float size = 0.5f * powf(sp[0] * sp[1] * sp[2], 1.0f / 3.0f) / (float)m;
  const size_t pts = capacity(g);
  float* dev = NULL;
  float scale = 0.0f;
  if (use_vortons) {
    dev = (float*)calloc(pts, sizeof(float));
    for (size_t i = 0; i < nv; ++i) accumulate1(g, dev, vpos + 3 * i, vdens[i] - ambient);
    float lo = FLT_MAX, hi = -FLT_MAX;
    for (size_t o = 0; o < pts; ++o) lo = minf_(dev[o], lo), hi = maxf_(dev[o], hi);
    scale = maxf_(fabsf(hi), fabsf(lo));
  }
  float shift[3], jm[3];
  const float jm_scale = 1.9999f * (1.0f - FLT_EPSILON);
  for (int a = 0; a < 3; ++a) {
    shift[a] = (0.5f * sp[a]) * (1.0f / (float)m);
    jm[a] = shift[a] * jm_scale;
  }
  size_t kept = 0;
  uint64_t d = 0;
  if (!use_vortons || scale != 0.0f) {
    const unsigned nc[3] = {g->np[0] - 1, g->np[1] - 1, g->np[2] - 1};
    unsigned idx[3], it[3];
    for (idx[2] = 0; idx[2] < nc[2]; ++idx[2])
      for (idx[1] = 0; idx[1] < nc[1]; ++idx[1])
        for (idx[0] = 0; idx[0] < nc[0]; ++idx[0]) {
          float cmin[3];
          for (int a = 0; a < 3; ++a) cmin[a] = g->mn[a] + (float)idx[a] * sp[a];
          for (it[2] = 0; it[2] < m; ++it[2])
            for (it[1] = 0; it[1] < m; ++it[1])
              for (it[0] = 0; it[0] < m; ++it[0]) {
                float j[3], p[3];
                spread3_(jm, host_rand, seed, &d, j);
                for (int a = 0; a < 3; ++a) p[a] = ((cmin[a] + ((float)it[a] / (float)m) * sp[a]) + shift[a]) + j[a];
                float dens = ambient;
                int emit = 1;
                if (use_vortons) {
                  float here;
                  interpolate_k(g, dev, 1, p, &here);
                  dens = (here + scale) * ambient;
                  emit = fabsf(here / scale) >= 0.5f;
                }
                if (emit) {
                  if (kept < max) {
                    memcpy(pos_out + 3 * kept, p, sizeof(p));
                    dens_out[kept] = dens;
                    size_out[kept] = size;
                  }
                  ++kept;
                }
              }
        }
  }
  free(dev);
  *count = kept;
}

/* PclOpEmit::Operate (pclOpEmit.cpp:188-210): emit int(dt x rate +
 * remainder) copies of the template, keeping the fraction in *remainder,
 * each varied by RandomSpread of the spread in the order position,
 * velocity, orientation, angular velocity, density, fuel, flame and smoke
 * fractions, size.  tmpl and spread hold those 17 values; per particle rec
 * receives them and the birth frame (as a float).  Returns the number
 * emitted (records written up to max). */
size_t vgo_emit_operate(const float tmpl[17], const float spread[17], float rate, float* remainder, float dt,
                        unsigned frame, int host_rand, unsigned seed, uint64_t* draw, float* rec, size_t max) {
  const float f = dt * rate + *remainder;
  const int k = (int)f;
  *remainder = f - (float)k;
  for (int i = 0; i < k; ++i) {
    float r[18];
    for (int v = 0; v < 4; ++v) {
      float s[3];
      spread3_(spread + 3 * v, host_rand, seed, draw, s);
      for (int a = 0; a < 3; ++a) r[3 * v + a] = tmpl[3 * v + a] + s[a];
    }
    for (int v = 12; v < 17; ++v) r[v] = tmpl[v] + spread_(spread[v], draw_(host_rand, seed, draw));
    r[17] = (float)(int)frame;
    if ((size_t)i < max) memcpy(rec + 18 * (size_t)i, r, sizeof(r));
  }
  return k > 0 ? (size_t)k : 0;
}
