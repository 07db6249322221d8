/*
 * CPU oracle for the spot-finder hot path. TEST INFRASTRUCTURE ONLY (see
 * sf_oracle.h): a plain-C restatement of src/spots/dext.cc and
 * src/spots/dials_spots.cc, used as the checker for the CUDA path.
 */
#include "sf_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

void or_default_params(or_params *p) {
  /* dext.cc:37-40 and :99, :203: kernel 3 (7 x 7), sigma_b 6, sigma_s 3,
   * gain 1 implied, at least 2 valid pixels, pixel above 0. */
  p->algorithm = OR_DISPERSION_EXTENDED;
  p->kernel_x = 3;
  p->kernel_y = 3;
  p->gain = 1.0;
  p->sigma_b = 6.0;
  p->sigma_s = 3.0;
  p->min_local = 2;
  p->global_threshold = 0.0;
}

/* Per-thread scratch of the threshold, grown as needed and kept for the
 * thread's life, as the reference's worker threads keep a thread_local
 * Scratch (src/spots/find_spots.cc:407-408, src/spots/dext.hh:49-74) instead
 * of allocating 26 bytes a pixel for every frame. Freed at thread exit. */
typedef struct {
  unsigned char *buf;
  size_t bytes;
} or_scratch;

static pthread_key_t g_scratch_key;
static pthread_once_t g_scratch_once = PTHREAD_ONCE_INIT;

static void or_scratch_free(void *p) {
  or_scratch *s = (or_scratch *)p;
  if (s) {
    free(s->buf);
    free(s);
  }
}

static void or_scratch_key_init(void) { pthread_key_create(&g_scratch_key, or_scratch_free); }

/* At least `bytes` of this thread's scratch, or NULL. */
static unsigned char *or_scratch_get(size_t bytes) {
  pthread_once(&g_scratch_once, or_scratch_key_init);
  or_scratch *s = (or_scratch *)pthread_getspecific(g_scratch_key);
  if (!s) {
    s = (or_scratch *)calloc(1, sizeof(or_scratch));
    if (!s || pthread_setspecific(g_scratch_key, s) != 0) {
      free(s);
      return NULL;
    }
  }
  if (s->bytes < bytes) {
    free(s->buf);
    s->buf = (unsigned char *)malloc(bytes);
    s->bytes = s->buf ? bytes : 0;
  }
  return s->buf;
}

#define OR_FN or_dext_u32
#define OR_T uint32_t
#define OR_W uint64_t
#define OR_R double
#define OR_SQRT sqrt
#define OR_TMAX 0xFFFFFFFFu
#include "sf_oracle_dext.inc"
#undef OR_FN
#undef OR_T
#undef OR_W
#undef OR_R
#undef OR_SQRT
#undef OR_TMAX

#define OR_FN or_dext_u16
#define OR_T uint16_t
#define OR_W uint32_t
#define OR_R float
#define OR_SQRT sqrtf
#define OR_TMAX 0xFFFFu
#include "sf_oracle_dext.inc"

/* ------------------------------------------------------------------------ */
/* 3-D labelling: a restatement of dials_spots::Labeller                     */
/* (src/spots/dials_spots.cc:36-360).                                        */
/* ------------------------------------------------------------------------ */

#define K_NONE 0xFFFFFFFFu
static const double kPixelVariance = 1.0 / 12.0; /* dials_spots.cc:14 */

typedef struct {
  void *data;
  size_t size, cap, elem;
} vec;

static int vec_reserve(vec *v, size_t n) {
  if (n <= v->cap)
    return 0;
  size_t cap = v->cap ? v->cap : 64;
  while (cap < n)
    cap *= 2;
  void *d = realloc(v->data, cap * v->elem);
  if (!d)
    return -1;
  v->data = d;
  v->cap = cap;
  return 0;
}
static int vec_resize(vec *v, size_t n) {
  if (vec_reserve(v, n))
    return -1;
  v->size = n;
  return 0;
}
#define VAT(v, T, i) (((T *)(v).data)[i])

struct or_labeller {
  size_t height, width, min_spot_size, max_spot_size;
  double max_separation;
  int two_d;
  vec live;   /* or_pixel */
  vec parent; /* uint32_t */
  size_t previous;
  int64_t last_frame;
  int started;
  vec spots; /* or_spot */
  vec kept;  /* or_pixel */
  or_counts counts;
  vec root, label, offset, cursor, member, open; /* scratch, as :150-157 */
};

or_labeller *or_label_open(size_t height, size_t width, size_t min_spot_size,
                           size_t max_spot_size, double max_separation,
                           int two_d) {
  /* dials_spots.cc:21-30 */
  if (height == 0 || width == 0 || max_spot_size < min_spot_size ||
      min_spot_size == 0)
    return NULL;
  or_labeller *l = (or_labeller *)calloc(1, sizeof(or_labeller));
  if (!l)
    return NULL;
  l->height = height;
  l->width = width;
  l->min_spot_size = min_spot_size;
  l->max_spot_size = max_spot_size;
  l->max_separation = max_separation;
  l->two_d = two_d;
  l->live.elem = sizeof(or_pixel);
  l->parent.elem = sizeof(uint32_t);
  l->spots.elem = sizeof(or_spot);
  l->kept.elem = sizeof(or_pixel);
  l->root.elem = l->label.elem = l->offset.elem = l->cursor.elem =
      l->member.elem = sizeof(uint32_t);
  l->open.elem = 1;
  return l;
}

void or_label_close(or_labeller *l) {
  if (!l)
    return;
  vec *all[] = {&l->live,   &l->parent, &l->spots,  &l->kept,
                &l->root,   &l->label,  &l->offset, &l->cursor,
                &l->member, &l->open};
  for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); i++)
    free(all[i]->data);
  free(l);
}

/* dials_spots.cc:36-55: path halving; union toward the lower index. */
static uint32_t lfind(or_labeller *l, uint32_t i) {
  uint32_t *parent = (uint32_t *)l->parent.data;
  while (parent[i] != i) {
    parent[i] = parent[parent[i]];
    i = parent[i];
  }
  return i;
}
static void lmerge(or_labeller *l, uint32_t a, uint32_t b) {
  const uint32_t ra = lfind(l, a), rb = lfind(l, b);
  if (ra == rb)
    return;
  uint32_t *parent = (uint32_t *)l->parent.data;
  if (ra < rb)
    parent[rb] = ra;
  else
    parent[ra] = rb;
}

/* dials_spots.cc:221-360 */
static int lemit(or_labeller *l, const uint32_t *members, size_t n) {
  l->counts.groups++;
  if (n < l->min_spot_size) {
    l->counts.too_small++;
    return 0;
  }
  if (n > l->max_spot_size) {
    l->counts.too_large++;
    return 0;
  }
  const or_pixel *live = (const or_pixel *)l->live.data;
  const size_t width = l->width;
  or_spot spot;
  memset(&spot, 0, sizeof(spot));
  spot.n_signal = (uint32_t)n;

  double sum = 0.0, sum_sq = 0.0;
  double weighted[3] = {0.0, 0.0, 0.0};
  int32_t x0 = 0, x1 = 0, y0 = 0, y1 = 0, z0 = 0, z1 = 0;
  uint32_t peak_value = 0;
  double peak[3] = {0.0, 0.0, 0.0};
  for (size_t k = 0; k < n; k++) {
    const or_pixel *px = &live[members[k]];
    const int32_t x = (int32_t)(px->index % width);
    const int32_t y = (int32_t)(px->index / width);
    const int32_t z = px->frame;
    if (k == 0) {
      x0 = x, x1 = x + 1, y0 = y, y1 = y + 1, z0 = z, z1 = z + 1;
    } else {
      x0 = x < x0 ? x : x0;
      x1 = x + 1 > x1 ? x + 1 : x1;
      y0 = y < y0 ? y : y0;
      y1 = y + 1 > y1 ? y + 1 : y1;
      z0 = z < z0 ? z : z0;
      z1 = z + 1 > z1 ? z + 1 : z1;
    }
    const double value = (double)px->value;
    const double position[3] = {(double)x + 0.5, (double)y + 0.5,
                                (double)z + 0.5};
    sum += value;
    sum_sq += value * value;
    for (int axis = 0; axis < 3; axis++)
      weighted[axis] += value * position[axis];
    if (px->value > peak_value) {
      peak_value = px->value;
      peak[0] = position[0], peak[1] = position[1], peak[2] = position[2];
    }
  }
  spot.bbox[0] = x0, spot.bbox[1] = x1, spot.bbox[2] = y0;
  spot.bbox[3] = y1, spot.bbox[4] = z0, spot.bbox[5] = z1;
  spot.intensity = sum;
  spot.intensity_variance = sum;

  if (sum > 0.0) {
    for (int axis = 0; axis < 3; axis++)
      spot.position[axis] = weighted[axis] / sum;
    double delta_sq[3] = {0.0, 0.0, 0.0};
    for (size_t k = 0; k < n; k++) {
      const or_pixel *px = &live[members[k]];
      const double value = (double)px->value;
      const double position[3] = {(double)(px->index % width) + 0.5,
                                  (double)(px->index / width) + 0.5,
                                  (double)px->frame + 0.5};
      for (int axis = 0; axis < 3; axis++) {
        const double delta = position[axis] - spot.position[axis];
        delta_sq[axis] += value * delta * delta;
      }
    }
    if (sum * sum > sum_sq) {
      for (int axis = 0; axis < 3; axis++) {
        const double variance = delta_sq[axis] * sum / (sum * sum - sum_sq);
        spot.variance[axis] = variance / sum + kPixelVariance;
      }
    } else {
      for (int axis = 0; axis < 3; axis++)
        spot.variance[axis] = kPixelVariance;
    }
    if (spot.bbox[5] == spot.bbox[4] + 1)
      spot.position[2] = (double)spot.bbox[4] + 0.5;
  } else {
    spot.position[0] = (spot.bbox[1] + spot.bbox[0]) / 2.0;
    spot.position[1] = (spot.bbox[3] + spot.bbox[2]) / 2.0;
    spot.position[2] = (spot.bbox[5] + spot.bbox[4]) / 2.0;
  }

  if (l->max_separation > 0.0) {
    const double dx = peak[0] - spot.position[0];
    const double dy = peak[1] - spot.position[1];
    const double dz = peak[2] - spot.position[2];
    if (sqrt(dx * dx + dy * dy + dz * dz) > l->max_separation) {
      l->counts.separated++;
      return 0;
    }
  }

  spot.first = l->kept.size;
  if (vec_reserve(&l->kept, l->kept.size + n) ||
      vec_reserve(&l->spots, l->spots.size + 1))
    return -3;
  for (size_t k = 0; k < n; k++)
    VAT(l->kept, or_pixel, l->kept.size++) = live[members[k]];
  memcpy(&VAT(l->spots, or_spot, l->spots.size++), &spot, sizeof(spot));
  l->counts.accepted++;
  return 0;
}

/* dials_spots.cc:153-219 */
static int lflush(or_labeller *l, int64_t keep_frame) {
  const size_t n = l->live.size;
  if (n == 0) {
    l->previous = 0;
    return 0;
  }
  if (vec_resize(&l->root, n) || vec_resize(&l->label, n) ||
      vec_resize(&l->member, n))
    return -3;
  uint32_t *root = (uint32_t *)l->root.data;
  uint32_t *label = (uint32_t *)l->label.data;
  for (size_t i = 0; i < n; i++)
    label[i] = K_NONE;
  uint32_t components = 0;
  for (size_t i = 0; i < n; i++) {
    const uint32_t r = lfind(l, (uint32_t)i);
    if (label[r] == K_NONE)
      label[r] = components++;
    root[i] = label[r];
  }

  if (vec_resize(&l->offset, (size_t)components + 1) ||
      vec_resize(&l->cursor, (size_t)components + 1) ||
      vec_resize(&l->open, components))
    return -3;
  uint32_t *offset = (uint32_t *)l->offset.data;
  uint32_t *cursor = (uint32_t *)l->cursor.data;
  uint32_t *member = (uint32_t *)l->member.data;
  char *open = (char *)l->open.data;
  memset(offset, 0, ((size_t)components + 1) * sizeof(uint32_t));
  for (size_t i = 0; i < n; i++)
    offset[root[i] + 1]++;
  for (size_t c = 0; c < components; c++)
    offset[c + 1] += offset[c];
  for (size_t c = 0; c < components; c++)
    cursor[c] = offset[c];
  for (size_t i = 0; i < n; i++)
    member[cursor[root[i]]++] = (uint32_t)i;

  memset(open, 0, components);
  const or_pixel *live = (const or_pixel *)l->live.data;
  for (size_t i = 0; i < n; i++)
    if (live[i].frame == keep_frame)
      open[root[i]] = 1;

  for (uint32_t c = 0; c < components; c++)
    if (!open[c])
      if (lemit(l, &member[offset[c]], offset[c + 1] - offset[c]))
        return -3;

  for (uint32_t c = 0; c < components; c++)
    cursor[c] = K_NONE;
  or_pixel *livew = (or_pixel *)l->live.data;
  uint32_t *parent = (uint32_t *)l->parent.data;
  size_t write = 0;
  for (size_t i = 0; i < n; i++) {
    const uint32_t c = root[i];
    if (!open[c])
      continue;
    if (cursor[c] == K_NONE)
      cursor[c] = (uint32_t)write;
    livew[write] = livew[i];
    parent[write] = cursor[c];
    write++;
  }
  l->live.size = write;
  l->parent.size = write;
  l->previous = write;
  while (l->previous > 0 && livew[l->previous - 1].frame == keep_frame)
    l->previous--;
  return 0;
}

/* dials_spots.cc:57-145 */
int or_label_add(or_labeller *l, int64_t frame, const or_signal_pixel *signal,
                 size_t count) {
  if (l->started && frame <= l->last_frame)
    return -1;
  if (l->started && frame != l->last_frame + 1)
    if (lflush(l, frame))
      return -3;

  const size_t pixels = l->height * l->width;
  const size_t base = l->live.size;
  const uint32_t columns = (uint32_t)l->width;
  if (base + count > (size_t)K_NONE)
    return -3;
  if (vec_reserve(&l->live, base + count) ||
      vec_reserve(&l->parent, base + count))
    return -3;
  for (size_t s = 0; s < count; s++) {
    if (signal[s].index >= pixels)
      return -2;
    if (l->live.size > base &&
        signal[s].index <= VAT(l->live, or_pixel, l->live.size - 1).index)
      return -2;
    or_pixel held;
    held.frame = (int32_t)frame;
    held.index = signal[s].index;
    held.value = signal[s].value;
    VAT(l->parent, uint32_t, l->parent.size++) = (uint32_t)l->live.size;
    VAT(l->live, or_pixel, l->live.size++) = held;
  }
  l->counts.signal_pixels += count;
  const size_t end = l->live.size;
  const or_pixel *live = (const or_pixel *)l->live.data;

  /* Left neighbour in the same row (:106-110). */
  for (size_t i = base + 1; i < end; i++)
    if (live[i].index % columns != 0 && live[i].index == live[i - 1].index + 1)
      lmerge(l, (uint32_t)i, (uint32_t)(i - 1));

  /* The pixel above (:115-123). */
  for (size_t i = base, up = base; i < end; i++) {
    if (live[i].index < columns)
      continue;
    const uint32_t target = live[i].index - columns;
    while (up < i && live[up].index < target)
      up++;
    if (up < i && live[up].index == target)
      lmerge(l, (uint32_t)i, (uint32_t)up);
  }

  /* The same pixel on the previous frame (:128-137). */
  if (!l->two_d && l->started && l->last_frame + 1 == frame &&
      l->previous < base) {
    for (size_t i = base, back = l->previous; i < end; i++) {
      const uint32_t target = live[i].index;
      while (back < base && live[back].index < target)
        back++;
      if (back < base && live[back].index == target)
        lmerge(l, (uint32_t)i, (uint32_t)back);
    }
  }

  l->started = 1;
  l->last_frame = frame;
  return lflush(l, l->two_d ? frame + 1 : frame) ? -3 : 0;
}

void or_label_finish(or_labeller *l) {
  if (!l->started)
    return;
  lflush(l, l->last_frame + 1);
}

size_t or_label_n_spots(const or_labeller *l) { return l->spots.size; }
size_t or_label_n_pixels(const or_labeller *l) { return l->kept.size; }
const or_spot *or_label_spots(const or_labeller *l) {
  return (const or_spot *)l->spots.data;
}
const or_pixel *or_label_pixels(const or_labeller *l) {
  return (const or_pixel *)l->kept.data;
}
void or_label_counts(const or_labeller *l, or_counts *out) { *out = l->counts; }
