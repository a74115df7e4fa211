/*
 * scenes.c -- seeded synthetic scenes and ray sets for the benchmark
 * workloads (libmrg_scenes.so).
 *
 * Every value is produced with IEEE basic operations only (+ - * / sqrt, in
 * double, rounded once to float) and an integer hash, so the same seed gives
 * bit-identical geometry and rays on x86-64 and aarch64.  Build with
 * -ffp-contract=off.
 *
 * Workloads (sizes follow the benchmark configurations):
 *   - icosphere: 20 * 4^level triangles, each icosahedron face split into an
 *     n x n triangular grid (n = 2^level), vertices projected to the sphere
 *     and displaced along the normal by 3-octave value noise;
 *   - instance field: rigid transforms (random rotation + jittered grid
 *     translation) inside a cube;
 *   - primary rays: pinhole camera, one jittered ray per pixel;
 *   - bounce rays: one cosine-weighted diffuse ray from each primary hit.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>

typedef struct { float pos[3]; float tMin; float dir[3]; float tMax; } scn_ray;

/* lowbias32 integer hash (C. Wellons). */
static inline uint32_t hash32(uint32_t x)
{
    x ^= x >> 16; x *= 0x7feb352dU;
    x ^= x >> 15; x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
static inline uint32_t hash3(uint32_t a, uint32_t b, uint32_t c)
{
    return hash32(a ^ hash32(b ^ hash32(c)));
}
/* uniform double in [0, 1) from 32 bits */
static inline double u01(uint32_t h) { return (double)h * (1.0 / 4294967296.0); }

typedef struct { uint32_t s; } rng_t;
static inline double rng_next(rng_t* r)
{
    r->s = hash32(r->s + 0x9E3779B9u);
    return u01(r->s);
}

/* ---------------------------------------------------------------------- */
/* value noise                                                             */
/* ---------------------------------------------------------------------- */
static inline double lattice(int32_t x, int32_t y, int32_t z, uint32_t seed)
{
    uint32_t h = hash3((uint32_t)x * 73856093u, (uint32_t)y * 19349663u ^ seed,
                       (uint32_t)z * 83492791u + seed);
    return u01(h) * 2.0 - 1.0;
}
static inline double smooth(double t) { return t * t * (3.0 - 2.0 * t); }

static double value_noise(double x, double y, double z, uint32_t seed)
{
    double fx = floor(x), fy = floor(y), fz = floor(z);
    int32_t ix = (int32_t)fx, iy = (int32_t)fy, iz = (int32_t)fz;
    double tx = smooth(x - fx), ty = smooth(y - fy), tz = smooth(z - fz);
    double c[2][2][2];
    for(int a = 0; a < 2; a++)
        for(int b = 0; b < 2; b++)
            for(int d = 0; d < 2; d++)
                c[a][b][d] = lattice(ix + a, iy + b, iz + d, seed);
    double x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * tx;
    double x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * tx;
    double x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * tx;
    double x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * tx;
    double y0 = x00 + (x10 - x00) * ty;
    double y1 = x01 + (x11 - x01) * ty;
    return y0 + (y1 - y0) * tz;
}

/* 3 octaves, frequency doubling, amplitude halving; result in ~[-1, 1]. */
static double fbm3(double x, double y, double z, uint32_t seed)
{
    double s = 0.0, amp = 1.0, f = 1.0, norm = 0.0;
    for(int o = 0; o < 3; o++)
    {
        s += amp * value_noise(x * f, y * f, z * f, seed + 101u * (uint32_t)o);
        norm += amp;
        amp *= 0.5; f *= 2.0;
    }
    return s / norm;
}

/* ---------------------------------------------------------------------- */
/* icosphere                                                               */
/* ---------------------------------------------------------------------- */
static const int ICO_F[20][3] = {
    {0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11},
    {1, 5, 9}, {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
    {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8}, {3, 8, 9},
    {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}
};

void mrgs_icosphere_counts(uint32_t level, uint32_t* nv, uint32_t* nt)
{
    uint64_t n = 1ull << level;
    if(nv) *nv = (uint32_t)(20ull * (n + 1) * (n + 2) / 2);
    if(nt) *nt = (uint32_t)(20ull * n * n);
}

/* Fills pos (3*nv floats) and idx (3*nt).  noise_freq scales the unit-sphere
 * point before the noise lookup.  Returns 0 on success. */
int mrgs_icosphere(uint32_t level, double radius, double noise_amp, double noise_freq,
                   uint32_t seed, float* pos, uint32_t* idx)
{
    if(level > 12) return -1;
    const double phi = (1.0 + sqrt(5.0)) * 0.5;
    double V[12][3] = {
        {-1, phi, 0}, {1, phi, 0}, {-1, -phi, 0}, {1, -phi, 0},
        {0, -1, phi}, {0, 1, phi}, {0, -1, -phi}, {0, 1, -phi},
        {phi, 0, -1}, {phi, 0, 1}, {-phi, 0, -1}, {-phi, 0, 1}
    };
    for(int i = 0; i < 12; i++)
    {
        double l = sqrt(V[i][0] * V[i][0] + V[i][1] * V[i][1] + V[i][2] * V[i][2]);
        V[i][0] /= l; V[i][1] /= l; V[i][2] /= l;
    }
    const uint32_t n = 1u << level;
    const uint32_t perFace = (n + 1) * (n + 2) / 2;
    uint64_t tcount = 0;
    for(int f = 0; f < 20; f++)
    {
        int a = ICO_F[f][0], b = ICO_F[f][1], c = ICO_F[f][2];
        /* make the winding outward (counter-clockwise seen from outside) */
        double e1[3], e2[3], nn[3], cc[3];
        for(int k = 0; k < 3; k++)
        {
            e1[k] = V[b][k] - V[a][k];
            e2[k] = V[c][k] - V[a][k];
            cc[k] = V[a][k] + V[b][k] + V[c][k];
        }
        nn[0] = e1[1] * e2[2] - e1[2] * e2[1];
        nn[1] = e1[2] * e2[0] - e1[0] * e2[2];
        nn[2] = e1[0] * e2[1] - e1[1] * e2[0];
        if(nn[0] * cc[0] + nn[1] * cc[1] + nn[2] * cc[2] < 0.0) { int t = b; b = c; c = t; }
        const uint32_t vbase = (uint32_t)f * perFace;
        /* vertex (i, j): weights (n-i-j) A + i B + j C, row-major over i */
        uint32_t vi = vbase;
        for(uint32_t i = 0; i <= n; i++)
            for(uint32_t j = 0; j <= n - i; j++)
            {
                double wa = (double)(n - i - j), wb = (double)i, wc = (double)j;
                double p[3];
                for(int k = 0; k < 3; k++)
                    p[k] = ((V[a][k] * wa + V[b][k] * wb) + V[c][k] * wc) / (double)n;
                double l = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
                for(int k = 0; k < 3; k++) p[k] /= l;
                double d = fbm3(p[0] * noise_freq, p[1] * noise_freq, p[2] * noise_freq, seed);
                double r = radius * (1.0 + noise_amp * d);
                for(int k = 0; k < 3; k++) pos[3ull * vi + k] = (float)(p[k] * r);
                vi++;
            }
        /* row start of i: sum_{r<i} (n + 1 - r) */
#define VID(ii, jj) (vbase + (ii) * (n + 1) - ((ii) * ((ii) - 1)) / 2 + (jj))
        for(uint32_t i = 0; i < n; i++)
            for(uint32_t j = 0; j < n - i; j++)
            {
                uint32_t* t = &idx[3ull * tcount++];
                t[0] = VID(i, j); t[1] = VID(i + 1, j); t[2] = VID(i, j + 1);
                if(i + j + 1 < n)
                {
                    t = &idx[3ull * tcount++];
                    t[0] = VID(i + 1, j); t[1] = VID(i + 1, j + 1); t[2] = VID(i, j + 1);
                }
            }
#undef VID
    }
    return (tcount == 20ull * n * n) ? 0 : -2;
}

/* ---------------------------------------------------------------------- */
/* instances                                                               */
/* ---------------------------------------------------------------------- */
/* Rotation Rz(b) * Ry(a) with (cos, sin) pairs from the rational
 * parametrisation c = (1 - t^2) / (1 + t^2), s = 2t / (1 + t^2), t uniform in
 * [-1, 1] (angles uniform-ish in (-180, 180] degrees, basic operations only).
 * For this family m0*m6 - m2*m4 = 0 in exact arithmetic. */
static void random_rotation(rng_t* r, double R[9])
{
    double ta = rng_next(r) * 2.0 - 1.0, tb = rng_next(r) * 2.0 - 1.0;
    double ca = (1.0 - ta * ta) / (1.0 + ta * ta), sa = 2.0 * ta / (1.0 + ta * ta);
    double cb = (1.0 - tb * tb) / (1.0 + tb * tb), sb = 2.0 * tb / (1.0 + tb * tb);
    /* Rz(b) = [[cb,-sb,0],[sb,cb,0],[0,0,1]], Ry(a) = [[ca,0,sa],[0,1,0],[-sa,0,ca]] */
    R[0] = cb * ca; R[1] = -sb; R[2] = cb * sa;
    R[3] = sb * ca; R[4] = cb;  R[5] = sb * sa;
    R[6] = -sa;     R[7] = 0.0; R[8] = ca;
}

/* `count` rigid transforms on a jittered cubic grid filling [-box/2, box/2]^3
 * (grid side = ceil(cbrt(count))), random rotations.  m34 row-major. */
int mrgs_instance_field(uint32_t count, uint32_t seed, double box, double jitter, float* m34)
{
    uint32_t side = 1;
    while(side * side * side < count) side++;
    double cell = box / (double)side;
    rng_t r = { hash32(seed ^ 0xA511E9B3u) };
    for(uint32_t i = 0; i < count; i++)
    {
        uint32_t gx = i % side, gy = (i / side) % side, gz = i / (side * side);
        double R[9];
        random_rotation(&r, R);
        double t[3];
        uint32_t g[3] = { gx, gy, gz };
        for(int k = 0; k < 3; k++)
            t[k] = -box * 0.5 + cell * ((double)g[k] + 0.5) + (rng_next(&r) * 2.0 - 1.0) * jitter;
        for(int row = 0; row < 3; row++)
        {
            for(int col = 0; col < 3; col++) m34[12ull * i + 4 * row + col] = (float)R[3 * row + col];
            m34[12ull * i + 4 * row + 3] = (float)t[row];
        }
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* rays                                                                    */
/* ---------------------------------------------------------------------- */
static void normalize3(double v[3])
{
    double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l; v[1] /= l; v[2] /= l;
}
static void cross3d(const double a[3], const double b[3], double o[3])
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* One jittered pinhole ray per pixel, row-major, tMin 0, tMax FLT_MAX. */
int mrgs_primary_rays(uint32_t w, uint32_t h, const double eye[3], const double target[3],
                      const double up[3], double tan_half_fov_y, uint32_t seed, scn_ray* out)
{
    double f[3] = { target[0] - eye[0], target[1] - eye[1], target[2] - eye[2] };
    normalize3(f);
    double rt[3], u[3];
    cross3d(f, up, rt); normalize3(rt);
    cross3d(rt, f, u);
    double aspect = (double)w / (double)h;
    for(uint32_t y = 0; y < h; y++)
        for(uint32_t x = 0; x < w; x++)
        {
            uint64_t i = (uint64_t)y * w + x;
            uint32_t hh = hash3((uint32_t)i, seed, 0x5eed1234u);
            double jx = u01(hh), jy = u01(hash32(hh));
            double sx = (((double)x + jx) / (double)w * 2.0 - 1.0) * tan_half_fov_y * aspect;
            double sy = (1.0 - ((double)y + jy) / (double)h * 2.0) * tan_half_fov_y;
            double d[3];
            for(int k = 0; k < 3; k++) d[k] = f[k] + rt[k] * sx + u[k] * sy;
            normalize3(d);
            scn_ray* r = &out[i];
            for(int k = 0; k < 3; k++) { r->pos[k] = (float)eye[k]; r->dir[k] = (float)d[k]; }
            r->tMin = 0.0f;
            r->tMax = 3.402823466e+38f;
        }
    return 0;
}

/* Bounce rays.  For each primary ray i with hit_inst[i] != ~0u: origin =
 * primary origin + t * dir, pushed 2e-4 along the geometric normal that faces
 * the incoming ray; direction cosine-distributed about that normal
 * (normalize(n + s), s uniform on the unit sphere).  Writes the compacted
 * rays to out and the source primary index to src (optional).  Returns the
 * number of bounce rays. */
uint32_t mrgs_bounce_rays(uint32_t n, const scn_ray* primary, const uint32_t* hit_inst,
                          const uint32_t* hit_prim, const float* hit_t,
                          const float* pos, const uint32_t* idx, const float* m34,
                          uint32_t seed, scn_ray* out, uint32_t* src)
{
    uint32_t m = 0;
    for(uint32_t i = 0; i < n; i++)
    {
        if(hit_inst[i] == 0xFFFFFFFFu) continue;
        const float* M = &m34[12ull * hit_inst[i]];
        const uint32_t* t = &idx[3ull * hit_prim[i]];
        double v[3][3];
        for(int c = 0; c < 3; c++)
            for(int k = 0; k < 3; k++) v[c][k] = pos[3ull * t[c] + k];
        double e1[3] = { v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2] };
        double e2[3] = { v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2] };
        double nl[3], nw[3];
        cross3d(e1, e2, nl);
        for(int r = 0; r < 3; r++) nw[r] = M[4 * r] * nl[0] + M[4 * r + 1] * nl[1] + M[4 * r + 2] * nl[2];
        normalize3(nw);
        const scn_ray* p = &primary[i];
        double dd = nw[0] * p->dir[0] + nw[1] * p->dir[1] + nw[2] * p->dir[2];
        if(dd > 0.0) { nw[0] = -nw[0]; nw[1] = -nw[1]; nw[2] = -nw[2]; }
        double o[3];
        for(int k = 0; k < 3; k++) o[k] = (double)p->pos[k] + (double)hit_t[i] * (double)p->dir[k] + 2e-4 * nw[k];
        rng_t r = { hash3(i, seed, 0xB0B0CAFEu) };
        double d[3], l2;
        for(;;)
        {
            double s[3];
            do
            {
                for(int k = 0; k < 3; k++) s[k] = rng_next(&r) * 2.0 - 1.0;
                l2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
            } while(l2 > 1.0 || l2 < 1e-4);
            double l = sqrt(l2);
            for(int k = 0; k < 3; k++) d[k] = nw[k] + s[k] / l;
            double dl2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if(dl2 > 1e-8) break;
        }
        normalize3(d);
        scn_ray* q = &out[m];
        for(int k = 0; k < 3; k++) { q->pos[k] = (float)o[k]; q->dir[k] = (float)d[k]; }
        q->tMin = 0.0f;
        q->tMax = 3.402823466e+38f;
        if(src) src[m] = i;
        m++;
    }
    return m;
}

/* Shadow rays from hit points towards a fixed light point: origin = bounce
 * ray origin, direction = light - origin (unnormalised), tMax = 1 (segment). */
uint32_t mrgs_shadow_rays(uint32_t n, const scn_ray* origins, const double light[3], scn_ray* out)
{
    for(uint32_t i = 0; i < n; i++)
    {
        scn_ray* q = &out[i];
        for(int k = 0; k < 3; k++)
        {
            q->pos[k] = origins[i].pos[k];
            q->dir[k] = (float)(light[k] - (double)origins[i].pos[k]);
        }
        q->tMin = 0.0f;
        q->tMax = 1.0f;
    }
    return n;
}
