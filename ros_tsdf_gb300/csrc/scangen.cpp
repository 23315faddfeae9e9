// Seeded synthetic lidar scans for tests and benchmarks.
//
// Scenes are a ground plane z = 0 over a square, axis-aligned boxes standing
// on the ground and spheres resting on it.  Scans are ray-cast analytically
// from a spinning multi-channel lidar (channels evenly spaced in elevation,
// azimuths evenly spaced over 360 degrees around the sensor heading), with
// Gaussian noise added to the range; rays that hit nothing within the maximum
// range are dropped.  Output is float32 world-frame xyz.
//
// Random numbers: SplitMix64 (G. Steele, D. Lea, C. Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014) as a counter-based hash, and
// the Box-Muller transform for Gaussian noise.  Every ray draws its noise from
// a hash of (seed, scan index, ray index), so a scan is the same whatever the
// thread count.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

inline double u01(uint64_t x) { return (double)(splitmix64(x) >> 11) * (1.0 / 9007199254740992.0); }

struct Stream {
  uint64_t s;
  double uniform() {
    s += 0x9E3779B97F4A7C15ull;
    return u01(s);
  }
  double range(double a, double b) { return a + (b - a) * uniform(); }
};

struct Box {
  double lo[3], hi[3];
};
struct Sphere {
  double c[3], r;
};

struct Scene {
  double half;
  std::vector<Box> boxes;
  std::vector<Sphere> spheres;
};

// Nearest hit t > 1e-6 along o + t d, or +inf.
double cast(const Scene& sc, const double o[3], const double d[3], double tmax) {
  double best = tmax;
  // ground plane over the square
  if (d[2] < 0.0) {
    double t = -o[2] / d[2];
    if (t > 1e-6 && t < best) {
      double x = o[0] + t * d[0], y = o[1] + t * d[1];
      if (std::fabs(x) <= sc.half && std::fabs(y) <= sc.half) best = t;
    }
  }
  for (const Box& b : sc.boxes) {
    double t0 = -1e300, t1 = 1e300;
    bool miss = false;
    for (int a = 0; a < 3; ++a) {
      if (d[a] == 0.0) {
        if (o[a] < b.lo[a] || o[a] > b.hi[a]) {
          miss = true;
          break;
        }
        continue;
      }
      double inv = 1.0 / d[a];
      double ta = (b.lo[a] - o[a]) * inv, tb = (b.hi[a] - o[a]) * inv;
      if (ta > tb) std::swap(ta, tb);
      if (ta > t0) t0 = ta;
      if (tb < t1) t1 = tb;
      if (t0 > t1) {
        miss = true;
        break;
      }
    }
    if (miss) continue;
    double t = t0 > 1e-6 ? t0 : t1;
    if (t > 1e-6 && t < best) best = t;
  }
  for (const Sphere& s : sc.spheres) {
    double oc[3] = {o[0] - s.c[0], o[1] - s.c[1], o[2] - s.c[2]};
    double b = oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2];
    double c = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - s.r * s.r;
    double disc = b * b - c;
    if (disc < 0.0) continue;
    double q = std::sqrt(disc);
    double t = -b - q;
    if (t <= 1e-6) t = -b + q;
    if (t > 1e-6 && t < best) best = t;
  }
  return best;
}

}  // namespace

extern "C" {

typedef struct {
  double half_extent;  // ground square is [-h, h]^2
  int n_boxes;
  double box_lo, box_hi;  // side lengths, uniform per axis
  int n_spheres;
  double sphere_lo, sphere_hi;  // radii
  uint64_t seed;
} sg_scene_cfg;

typedef struct {
  int channels, azimuths;
  double elev_lo_deg, elev_hi_deg;
  double max_range, sigma;
} sg_lidar_cfg;

typedef struct {
  int kind;  // 0: circle of `radius` around the origin; 1: random walk
  double radius, height, speed, rate_hz;
  uint64_t seed;
} sg_traj_cfg;

void* sg_scene_create(const sg_scene_cfg* c) {
  Scene* s = new Scene();
  s->half = c->half_extent;
  Stream r{splitmix64(c->seed ^ 0x5CE4E5EEDull)};
  for (int i = 0; i < c->n_boxes; ++i) {
    Box b;
    double cx = r.range(-c->half_extent, c->half_extent), cy = r.range(-c->half_extent, c->half_extent);
    double sx = r.range(c->box_lo, c->box_hi), sy = r.range(c->box_lo, c->box_hi), sz = r.range(c->box_lo, c->box_hi);
    b.lo[0] = cx - sx / 2, b.hi[0] = cx + sx / 2;
    b.lo[1] = cy - sy / 2, b.hi[1] = cy + sy / 2;
    b.lo[2] = 0.0, b.hi[2] = sz;
    s->boxes.push_back(b);
  }
  for (int i = 0; i < c->n_spheres; ++i) {
    Sphere sp;
    sp.r = r.range(c->sphere_lo, c->sphere_hi);
    sp.c[0] = r.range(-c->half_extent, c->half_extent);
    sp.c[1] = r.range(-c->half_extent, c->half_extent);
    sp.c[2] = sp.r;
    s->spheres.push_back(sp);
  }
  return s;
}

void sg_scene_destroy(void* s) { delete (Scene*)s; }

// Sensor position and heading (radians) at scan k.
void sg_pose(const sg_traj_cfg* t, int k, double* pos3, double* yaw) {
  const double step = t->speed / t->rate_hz;
  if (t->kind == 0) {
    double a = (double)k * step / t->radius;
    pos3[0] = t->radius * std::cos(a);
    pos3[1] = t->radius * std::sin(a);
    pos3[2] = t->height;
    *yaw = a + M_PI / 2;
    return;
  }
  // random walk: heading drifts by N(0, 0.2 rad) per scan, reflected at 80%
  // of `radius` (the half extent of the scene)
  double x = 0, y = 0, h = 0;
  for (int i = 0; i < k; ++i) {
    uint64_t key = splitmix64(t->seed * 1000003ull + (uint64_t)i);
    double u1 = std::max(u01(key), 1e-300), u2 = u01(key ^ 0xABCDEFull);
    h += 0.2 * std::sqrt(-2.0 * std::log(u1)) * std::cos(2 * M_PI * u2);
    double nx = x + step * std::cos(h), ny = y + step * std::sin(h);
    double lim = 0.8 * t->radius;
    if (std::fabs(nx) > lim || std::fabs(ny) > lim) {
      h += M_PI;
      nx = x + step * std::cos(h);
      ny = y + step * std::sin(h);
    }
    x = nx, y = ny;
  }
  pos3[0] = x, pos3[1] = y, pos3[2] = t->height;
  *yaw = h;
}

// Cast one scan.  Writes up to `cap` points (xyz float32) and returns the
// number of hits.
int64_t sg_scan(void* scene, const sg_lidar_cfg* l, const double origin[3], double yaw, uint64_t noise_seed,
                int scan_idx, float* out_xyz, int64_t cap, int nthreads) {
  const Scene& sc = *(Scene*)scene;
  const int64_t nrays = (int64_t)l->channels * l->azimuths;
  std::vector<float> buf((size_t)nrays * 3);
  std::vector<uint8_t> hit((size_t)nrays, 0);
  if (nthreads < 1) nthreads = 1;
  auto work = [&](int64_t a, int64_t b) {
    for (int64_t r = a; r < b; ++r) {
      int ch = (int)(r / l->azimuths), az = (int)(r % l->azimuths);
      double el = l->channels > 1
                      ? l->elev_lo_deg + (l->elev_hi_deg - l->elev_lo_deg) * (double)ch / (double)(l->channels - 1)
                      : l->elev_lo_deg;
      el *= M_PI / 180.0;
      double azr = yaw + 2.0 * M_PI * (double)az / (double)l->azimuths;
      double d[3] = {std::cos(el) * std::cos(azr), std::cos(el) * std::sin(azr), std::sin(el)};
      double t = cast(sc, origin, d, l->max_range);
      if (!(t < l->max_range)) continue;
      uint64_t key = splitmix64(noise_seed ^ splitmix64(((uint64_t)(uint32_t)scan_idx << 32) | (uint64_t)r));
      double u1 = std::max(u01(key), 1e-300), u2 = u01(key ^ 0x1234567ull);
      double n = l->sigma * std::sqrt(-2.0 * std::log(u1)) * std::cos(2 * M_PI * u2);
      double rr = t + n;
      if (rr <= 0.0) continue;
      buf[3 * r] = (float)(origin[0] + rr * d[0]);
      buf[3 * r + 1] = (float)(origin[1] + rr * d[1]);
      buf[3 * r + 2] = (float)(origin[2] + rr * d[2]);
      hit[r] = 1;
    }
  };
  std::vector<std::thread> th;
  int64_t per = (nrays + nthreads - 1) / nthreads;
  for (int i = 0; i < nthreads; ++i) {
    int64_t a = i * per, b = std::min<int64_t>(nrays, a + per);
    if (a < b) th.emplace_back(work, a, b);
  }
  for (auto& t : th) t.join();
  int64_t n = 0;
  for (int64_t r = 0; r < nrays; ++r) {
    if (!hit[r]) continue;
    if (n < cap) std::memcpy(out_xyz + 3 * n, &buf[3 * r], 3 * sizeof(float));
    ++n;
  }
  return n;
}

}  // extern "C"
