/*
 * mcvox_kernel.cuh - photon-packet transport in a voxelized sample
 * (the GB300 counterpart of McKernel, xopto/mcvox/kernel/mcvox.template.c:548-1048).
 *
 * Same thread/stream mapping and run control as the layered kernel.  Each
 * step moves the packet by min(free path, distance to the current voxel's
 * wall).  Voxels are stored as one uint8 material index each (the reference
 * uses a 4-byte McVoxel, xopto/mcvox/mcgeometry/voxel.py:33-85), read through
 * the read-only data cache; the material table lives in shared memory.
 */
#pragma once
#include "mc_device.cuh"
#include "batch_rng.h"

namespace MCGB_NS {

/* Shared-memory record of one material. */
struct __align__(16) MvMaterial {
    float4 g0;    /* mus, mua, step_factor(inv_mut), mua_inv_mut */
    float4 g1;    /* n, -, -, - */
    float4 pf0;   /* phase-function constants (pf_prepare) */
    float4 pf1;
};

struct MvSmem {
    MvMaterial materials[MCGB_MAX_MATERIALS];
};

struct MvGeom {
    float tl[3], br[3], vs[3];
    int sh[3];
};

static __device__ __forceinline__ bool mv_valid(const MvGeom &g, const i3 &i) {
    return i.x >= 0 && i.x < g.sh[0] && i.y >= 0 && i.y < g.sh[1] && i.z >= 0 && i.z < g.sh[2];
}
/* mcsim_flat_voxel_index, xopto/mcvox/kernel/mcvox.template.h:786-804 */
static __device__ __forceinline__ int mv_material_at(const MvGeom &g, const uint8_t *vox, const i3 &i) {
    uint64_t flat = ((uint64_t)i.z * (uint64_t)g.sh[1] + (uint64_t)i.y) * (uint64_t)g.sh[0] + (uint64_t)i.x;
    return __ldg(vox + flat);
}
/* mcsim_position_to_voxel_index, mcvox.template.c:206-220 */
static __device__ __forceinline__ i3 mv_index(const MvGeom &g, const f3 &p) {
    return i3{cvt_int(mc_div(p.x - g.tl[0], g.vs[0])), cvt_int(mc_div(p.y - g.tl[1], g.vs[1])),
              cvt_int(mc_div(p.z - g.tl[2], g.vs[2]))};
}

/* mcsim_sample_box_intersect, mcvox.template.c:94-162 */
static __device__ __forceinline__ int mv_box_intersect(const MvGeom &g, const f3 &pos, const f3 &dir,
                                                       f3 &isec, f3 &normal) {
    float ix = (dir.x != 0.0f) ? mc_div(1.0f, dir.x) : __int_as_float(0x7f800000);
    float iy = (dir.y != 0.0f) ? mc_div(1.0f, dir.y) : __int_as_float(0x7f800000);
    float iz = (dir.z != 0.0f) ? mc_div(1.0f, dir.z) : __int_as_float(0x7f800000);
    float t1 = (g.tl[0] - pos.x) * ix, t2 = (g.br[0] - pos.x) * ix;
    float t3 = (g.tl[1] - pos.y) * iy, t4 = (g.br[1] - pos.y) * iy;
    float t5 = (g.tl[2] - pos.z) * iz, t6 = (g.br[2] - pos.z) * iz;
    float txmin = fminf(t1, t2), txmax = fmaxf(t1, t2);
    float tymin = fminf(t3, t4), tymax = fmaxf(t3, t4);
    float tzmin = fminf(t5, t6), tzmax = fmaxf(t5, t6);
    float tmin = fmaxf(fmaxf(txmin, tymin), tzmin);
    float tmax = fminf(fminf(txmax, tymax), tzmax);
    if (tmin > tmax) return 0;
    normal.x = (float)(txmin >= tymin && txmin >= tzmin);
    normal.y = (float)((normal.x == 0.0f) && tymin >= tzmin);
    normal.z = (float)(normal.x == 0.0f && normal.y == 0.0f);
    normal.x *= (float)fsign(dir.x);
    normal.y *= (float)fsign(dir.y);
    normal.z *= (float)fsign(dir.z);
    float tt = (tmin > 0.0f) ? tmin : tmax;
    isec.x = pos.x + tt * dir.x;
    isec.y = pos.y + tt * dir.y;
    isec.z = pos.z + tt * dir.z;
    isec.x = fminf(fmaxf(isec.x, g.tl[0]), g.br[0] - 1.1920929e-07f);
    isec.y = fminf(fmaxf(isec.y, g.tl[1]), g.br[1] - 1.1920929e-07f);
    isec.z = fminf(fmaxf(isec.z, g.tl[2]), g.br[2] - 1.1920929e-07f);
    return tmax >= tmin && tmax >= 0.0f;
}

/* mcsim_sample_box_contains, xopto/mcvox/kernel/mcvox.template.h:1227-1235 */
static __device__ __forceinline__ bool mv_contains(const MvGeom &g, const f3 &p) {
    return p.x >= g.tl[0] && p.x < g.br[0] && p.y >= g.tl[1] && p.y < g.br[1] && p.z >= g.tl[2] &&
           p.z < g.br[2];
}

/* Refractive index of the voxel at a point on the box surface
   (mcsim_position_to_voxel_index_safe + material lookup). */
static __device__ __forceinline__ float mv_n_at_surface(const MvGeom &g, const MvMaterial *M,
                                                        const uint8_t *vox, const f3 &p) {
    i3 li = mv_index(g, p);
    li.x = clip_i(li.x, 0, g.sh[0] - 1);
    li.y = clip_i(li.y, 0, g.sh[1] - 1);
    li.z = clip_i(li.z, 0, g.sh[2] - 1);
    return M[mv_material_at(g, vox, li)].g1.x;
}

/* Entry of a collimated beam into the voxel box, shared by GaussianBeam
   (xopto/mcvox/mcsource/gaussianbeam.py:112-190) and UniformBeam
   (uniformbeam.py:104-186): from a point pm of the beam, move along the
   beam direction (backwards if pm lies inside the box) to the box surface,
   refract and weigh with the Fresnel reflectance; a beam that misses the
   box starts at the top-left corner with zero weight. */
static __device__ __forceinline__ void mv_beam_enter(const McgbMcvoxConfig &c, const MvGeom &g,
                                                     const MvMaterial *M, const uint8_t *vox,
                                                     f3 pm, f3 &pos, f3 &dir, float &w,
                                                     uint64_t *accu) {
    const McgbSource &src = c.source;
    float specular_r;
    f3 direction{src.direction[0], src.direction[1], src.direction[2]};
    if (mv_contains(g, pm)) direction = f3{-direction.x, -direction.y, -direction.z};
    f3 isec, normal;
    if (mv_box_intersect(g, pm, direction, isec, normal)) {
        pos = isec;
        direction = f3{-direction.x, -direction.y, -direction.z};
        normal = f3{-normal.x, -normal.y, -normal.z};
        float n_outside = M[0].g1.x;
        float n_inside = mv_n_at_surface(g, M, vox, pos);
        f3 refracted = direction;
        refract_safe3(direction, normal, n_outside, n_inside, &refracted);
        dir = refracted;
        specular_r = reflectance(n_outside, n_inside, dot3(normal, direction),
                                 cos_critical(n_outside, n_inside));
        if (c.specular.kind != MCGB_DET_NONE)
            detector_deposit(c.specular, pos, direction, specular_r, 0.0f, accu);
    } else {
        pos = f3{g.tl[0], g.tl[1], g.tl[2]};
        dir = f3{0.0f, 0.0f, 1.0f};
        specular_r = 1.0f;
    }
    w = 1.0f - specular_r;
}

/* Packet launch of the voxelized medium: Line (xopto/mcvox/mcsource/line.py),
   GaussianBeam (gaussianbeam.py:112-190), UniformBeam (uniformbeam.py:104-186),
   IsotropicPoint (point.py:74-140), UniformFiber / LambertianFiber
   (fiber.py:257-352,603-700) and IsotropicVoxel (voxel.py:78-107); then the
   voxel index of the launch position (mcvox.template.c:240-262). */
template <bool SIMPLE>
static __device__ __forceinline__ void mcvox_launch(const McgbMcvoxConfig &c, const MvGeom &g,
                                                    const MvMaterial *M, const uint8_t *vox,
                                                    const float *lut, Rng &rng, f3 &pos, f3 &dir,
                                                    float &w, i3 &vi, int &mat, uint64_t *accu,
                                                    f3 prev_pos) {
    const McgbSource &src = c.source;
    const float *T = src.transformation;
    if (src.kind == MCGB_SRC_LINE) {
        w = 1.0f - src.reflectance;
        pos = f3{src.position[0], src.position[1], src.position[2]};
        dir = f3{src.direction[0], src.direction[1], src.direction[2]};
        if (c.specular.kind != MCGB_DET_NONE) {
            f3 d{src.direction_reflected[0], src.direction_reflected[1], src.direction_reflected[2]};
            detector_deposit(c.specular, pos, d, src.reflectance, 0.0f, accu);
        }
    } else if (SIMPLE || src.kind == MCGB_SRC_GAUSSIAN_BEAM || src.kind == MCGB_SRC_UNIFORM_BEAM) {
        float sin_fi, cos_fi;
        f3 ps;
        if (SIMPLE || src.kind == MCGB_SRC_GAUSSIAN_BEAM) {
            float r = mc_sqrt(-2.0f * mc_log(1.0f - rng.next()));
            r = fminf(r, src.clip);
            mc_sincos(6.28318548f * rng.next(), &sin_fi, &cos_fi);
            ps = f3{r * cos_fi * src.sigma[0], r * sin_fi * src.sigma[1], 0.0f};
        } else {
            float rand_sqrt = mc_sqrt(rng.next());
            float fi = 6.28318548f * rng.next();
            mc_sincos(fi, &sin_fi, &cos_fi);
            ps = f3{rand_sqrt * cos_fi * src.sigma[0], rand_sqrt * sin_fi * src.sigma[1], 0.0f};
        }
        f3 pm{T[0] * ps.x + T[1] * ps.y + T[2] * ps.z,
              T[3] * ps.x + T[4] * ps.y + T[5] * ps.z,
              T[6] * ps.x + T[7] * ps.y + T[8] * ps.z};
        pm.x += src.position[0];
        pm.y += src.position[1];
        pm.z += src.position[2];
        mv_beam_enter(c, g, M, vox, pm, pos, dir, w, accu);
    } else if (src.kind == MCGB_SRC_ISOTROPIC_POINT) {
        /* Two quirks of the reference, restated: the refraction goes to a
           shadowing local variable, so the direction stays unrefracted
           (xopto/mcvox/mcsource/point.py:115-117); and the voxel lookup of
           n_inside reads the simulator's current position instead of the
           intersection (xopto/mcvox/kernel/mcvox.template.c:206-220), i.e.
           the previous packet's final position on the same stream (prev_pos;
           the origin for a stream's first packet and under dynamic
           scheduling, where a packet has no predecessor). */
        float sin_fi, cos_fi, specular_r = 0.0f;
        pos = f3{src.position[0], src.position[1], src.position[2]};
        mc_sincos(rng.next() * 6.28318548f, &sin_fi, &cos_fi);
        float cos_theta = 1.0f - 2.0f * rng.next();
        float sin_theta = mc_sqrt(1.0f - cos_theta * cos_theta);
        f3 d{cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
        if (!mv_contains(g, pos)) {
            f3 isec, normal;
            if (mv_box_intersect(g, pos, d, isec, normal)) {
                pos = isec;
                float n_outside = M[0].g1.x;
                float n_inside = mv_n_at_surface(g, M, vox, prev_pos);
                specular_r = reflectance(n_outside, n_inside, dot3(normal, d),
                                         cos_critical(n_outside, n_inside));
            } else {
                pos = f3{g.tl[0], g.tl[1], g.tl[2]};
                specular_r = 1.0f;
            }
        }
        dir = d;
        if (c.specular.kind != MCGB_DET_NONE) detector_deposit(c.specular, pos, d, specular_r, 0.0f, accu);
        w = 1.0f - specular_r;
    } else if (src.kind == MCGB_SRC_UNIFORM_FIBER || src.kind == MCGB_SRC_LAMBERTIAN_FIBER ||
               src.kind == MCGB_SRC_UNIFORM_FIBER_LUT) {
        /* UniformFiberLut samples the cosine from its emission LUT
           (xopto/mcvox/mcsource/fiber.py:843-845) */
        float sin_fi, cos_fi, sin_theta, cos_theta, specular_r;
        float r = mc_sqrt(rng.next()) * src.sigma[0];
        mc_sincos(rng.next() * 6.28318548f, &sin_fi, &cos_fi);
        f3 ps{r * cos_fi, r * sin_fi, 0.0f};
        f3 pm{T[0] * ps.x + T[1] * ps.y + T[2] * ps.z,
              T[3] * ps.x + T[4] * ps.y + T[5] * ps.z,
              T[6] * ps.x + T[7] * ps.y + T[8] * ps.z};
        pm.x += src.position[0];
        pm.y += src.position[1];
        pm.z += src.position[2];
        mc_sincos(rng.next() * 6.28318548f, &sin_fi, &cos_fi);
        if (src.kind == MCGB_SRC_LAMBERTIAN_FIBER) {
            sin_theta = mc_sqrt(rng.next()) * src.sigma[1];
        } else {
            cos_theta = src.kind == MCGB_SRC_UNIFORM_FIBER_LUT
                            ? lut_sample_rel(lut + src.lut_offset, src.lut_size, rng.next(), 0.0f)
                            : 1.0f - rng.next() * (1.0f - src.sigma[1]);
            sin_theta = mc_sqrt(1.0f - cos_theta * cos_theta);
        }
        sin_theta = mc_div(sin_theta, src.clip);
        cos_theta = mc_sqrt(1.0f - sin_theta * sin_theta);
        f3 pt{cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
        f3 packet_dir{T[0] * pt.x + T[1] * pt.y + T[2] * pt.z,
                      T[3] * pt.x + T[4] * pt.y + T[5] * pt.z,
                      T[6] * pt.x + T[7] * pt.y + T[8] * pt.z};
        f3 source_dir{src.direction[0], src.direction[1], src.direction[2]};
        if (mv_contains(g, pm)) source_dir = f3{-source_dir.x, -source_dir.y, -source_dir.z};
        f3 refracted = packet_dir;
        f3 isec, normal;
        if (mv_box_intersect(g, pm, source_dir, isec, normal)) {
            normal = f3{-normal.x, -normal.y, -normal.z};
            pos = isec;
            float n_outside = src.clip;
            float n_inside = mv_n_at_surface(g, M, vox, isec);
            refract_safe3(packet_dir, normal, n_outside, n_inside, &refracted);
            specular_r = reflectance(n_outside, n_inside, dot3(normal, packet_dir),
                                     cos_critical(n_outside, n_inside));
        } else {
            pos = f3{g.tl[0], g.tl[1], g.tl[2]};
            specular_r = 1.0f;
        }
        dir = refracted;
        if (c.specular.kind != MCGB_DET_NONE)
            detector_deposit(c.specular, pos, packet_dir, specular_r, 0.0f, accu);
        w = 1.0f - specular_r;
    } else {
        /* IsotropicVoxel(s): uniform in the voxel, isotropic direction;
           IsotropicVoxels first picks one of its voxels (voxel.py:230-245) */
        float vx = src.direction[0], vy = src.direction[1], vz = src.direction[2];
        w = 1.0f;
        if (src.kind == MCGB_SRC_ISOTROPIC_VOXELS) {
            int n = (int)src.lut_size;
            int k = min(cvt_int(rng.next() * (float)src.lut_size), n - 1);
            const float *e = lut + src.lut_offset + (size_t)k * 4u;
            w = e[0];
            vx = e[1];
            vy = e[2];
            vz = e[3];
        }
        const float one_minus_eps = 1.0f - 1.1920929e-07f;
        float ux = fminf(rng.next(), one_minus_eps);
        float px = (vx + ux) * g.vs[0] + g.tl[0];
        float uy = fminf(rng.next(), one_minus_eps);
        float py = (vy + uy) * g.vs[1] + g.tl[1];
        float uz = fminf(rng.next(), one_minus_eps);
        float pz = (vz + uz) * g.vs[2] + g.tl[2];
        pos = f3{px, py, pz};
        float sin_fi, cos_fi;
        mc_sincos(rng.next() * 6.28318548f, &sin_fi, &cos_fi);
        float cos_theta = 1.0f - 2.0f * rng.next();
        float sin_theta = mc_sqrt(1.0f - cos_theta * cos_theta);
        dir = f3{cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
    }
    vi = mv_index(g, pos);
    mat = mv_valid(g, vi) ? mv_material_at(g, vox, vi) : 0;
}

/* mcsim_boundary (mcvox), mcvox.template.c:275-388 */
static __device__ __forceinline__ uint32_t mv_boundary(const MvGeom &g, const MvMaterial *M,
                                                       const uint8_t *vox, f3 &dir, i3 &vi,
                                                       int &mat, const f3 &dist, Rng &rng) {
    i3 nrm;
    nrm.x = (dist.x <= dist.y) && (dist.x <= dist.z);
    nrm.y = nrm.x ? 0 : ((dist.y <= dist.x) && (dist.y <= dist.z));
    nrm.z = !(nrm.x + nrm.y);
    nrm.x = dir.x < 0.0f ? -nrm.x : nrm.x;
    nrm.y = dir.y < 0.0f ? -nrm.y : nrm.y;
    nrm.z = dir.z < 0.0f ? -nrm.z : nrm.z;
    i3 nv{vi.x + nrm.x, vi.y + nrm.y, vi.z + nrm.z};
    bool escaping = !mv_valid(g, nv);
    int next_mat = !escaping ? mv_material_at(g, vox, nv) : 0;
    if (mat == next_mat && !escaping) {
        vi = nv;
        return MCGB_EV_REFRACTION;
    }
    float n1 = M[mat].g1.x, n2 = M[next_mat].g1.x;
    if (n1 == n2) {
        vi = nv;
        mat = next_mat;
        return MCGB_EV_REFRACTION;
    }
    float cc = cos_critical(n1, n2);
    float cos1 = (float)nrm.x * dir.x + (float)nrm.y * dir.y + (float)nrm.z * dir.z;
    f3 fn{(float)nrm.x, (float)nrm.y, (float)nrm.z};
    if (cos1 > cc) {
        float R = reflectance(n1, n2, cos1, cc);
        if (R < rng.next()) {
            dir = refract3(dir, fn, n1, n2);
            vi = nv;
            mat = next_mat;
            return MCGB_EV_REFRACTION;
        }
    }
    dir = reflect3(dir, fn);
    return MCGB_EV_REFLECTION;
}

struct MvCtx {
    const MvMaterial *M;
    const float *lut;
    const uint8_t *vox;
    const uint8_t *rad;   /* homogeneous-cube radii (FAST free flight), or NULL */
    MvGeom g;
    float rmax2, rmax;
    float free_unit;      /* smallest voxel size, less a relative margin */
    float free_eps;       /* absolute margin for the rounding of positions */
    bool use_rmax, use_trace, track_opl;
    uint32_t max_steps;   /* per-packet step limit, 0xFFFFFFFF when unlimited */
    f3 src_pos;
};

struct MvPacket {
    f3 pos, dir;
    i3 vi;                /* the voxel; with free flight, the centre of the packet's cube */
    int mat;
    float w, opl;
    float free;           /* FAST: radius around pos inside the cube, 0 = none */
    int k;                /* FAST: half width of the cube around vi in voxels, 0 = the voxel */
    float pend;           /* phased loop: the sampled path not yet taken, < 0 = none */
    uint32_t trace_count, events, steps;
    uint64_t p;
};

/* True when the cube of half width k around vi lies inside the rmax sphere
   (with a relative margin): no position inside it ends a packet. */
static __device__ __forceinline__ bool mv_cube_in_rmax(const MvCtx &x, const i3 &vi, int k) {
    const MvGeom &g = x.g;
    const int v[3] = {vi.x, vi.y, vi.z};
    const float src[3] = {x.src_pos.x, x.src_pos.y, x.src_pos.z};
    float r2 = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float lo = g.tl[a] + (float)(v[a] - k) * g.vs[a] - src[a];
        float hi = g.tl[a] + (float)(v[a] + k + 1) * g.vs[a] - src[a];
        float m = fmaxf(fabsf(lo), fabsf(hi));
        r2 = fmaf(m, m, r2);
    }
    return r2 < x.rmax2 * 0.9999f;
}

/* Homogeneous-cube half width k of voxel vi (mcgb_voxel_radius): every
   voxel within Chebyshev distance k of vi lies inside the grid and holds
   vi's material.  With a finite rmax the cube also shrinks until it lies
   inside the rmax sphere.  0 when free flight is off or vi lies outside the
   grid. */
static __device__ __forceinline__ int mv_cube_k(const MvCtx &x, const i3 &vi) {
    if (!x.rad || !mv_valid(x.g, vi)) return 0;
    uint64_t flat = ((uint64_t)vi.z * (uint64_t)x.g.sh[1] + (uint64_t)vi.y) * (uint64_t)x.g.sh[0] +
                    (uint64_t)vi.x;
    int k = __ldg(x.rad + flat);
    if (x.use_rmax)
        while (k > 0 && !mv_cube_in_rmax(x, vi, k)) --k;
    return k;
}

/* Radius of a ball around any point of voxel vi inside its cube of half
   width k: k times the smallest voxel size, less the margins. */
static __device__ __forceinline__ float mv_ball(const MvCtx &x, int k) {
    return k == 0 ? 0.0f : fmaxf((float)k * x.free_unit - x.free_eps, 0.0f);
}

/* Radius of a ball around pos, a point of the cube of half width k around
   vi: its distance to the cube's faces, less the margins. */
static __device__ __forceinline__ float mv_clearance(const MvCtx &x, const i3 &vi, int k, const f3 &pos) {
    if (k == 0) return 0.0f;
    const MvGeom &g = x.g;
    float c = pos.x - (g.tl[0] + (float)(vi.x - k) * g.vs[0]);
    c = fminf(c, g.tl[0] + (float)(vi.x + k + 1) * g.vs[0] - pos.x);
    c = fminf(c, pos.y - (g.tl[1] + (float)(vi.y - k) * g.vs[1]));
    c = fminf(c, g.tl[1] + (float)(vi.y + k + 1) * g.vs[1] - pos.y);
    c = fminf(c, pos.z - (g.tl[2] + (float)(vi.z - k) * g.vs[2]));
    c = fminf(c, g.tl[2] + (float)(vi.z + k + 1) * g.vs[2] - pos.z);
    return fmaxf(c * 0.999f - x.free_eps, 0.0f);
}

static __device__ __forceinline__ MvCtx mcvox_ctx(const McgbMcvoxConfig &c, const McgbBuffers &b,
                                                  const MvMaterial *M, const float *lut) {
    MvCtx x;
    x.M = M;
    x.lut = lut;
    x.vox = b.voxels;
    for (int k = 0; k < 3; ++k) {
        x.g.tl[k] = c.top_left[k];
        x.g.br[k] = c.bottom_right[k];
        x.g.vs[k] = c.voxel_size[k];
        x.g.sh[k] = c.shape[k];
    }
    x.rmax = c.opt.rmax;
    x.rmax2 = c.opt.rmax * c.opt.rmax;
    x.use_rmax = x.rmax2 < __int_as_float(0x7f800000);
    x.use_trace = c.trace.flags != MCGB_TRACE_NONE;
    x.track_opl = c.opt.track_optical_pathlength != 0;
    x.max_steps = (c.opt.max_steps_per_packet == 0 || c.opt.max_steps_per_packet > 0xFFFFFFFFull)
                      ? 0xFFFFFFFFu : (uint32_t)c.opt.max_steps_per_packet;
    x.src_pos = f3{c.source.position[0], c.source.position[1], c.source.position[2]};
    /* Free flight (FAST math, no trace: a trace records every wall stop). */
    x.rad = (MCGB_FAST_MATH && !x.use_trace) ? b.voxel_radius : nullptr;
    x.free_unit = fminf(x.g.vs[0], fminf(x.g.vs[1], x.g.vs[2])) * 0.999f;
    float ext = 0.0f;
    for (int k = 0; k < 3; ++k) ext = fmaxf(ext, fmaxf(fabsf(x.g.tl[k]), fabsf(x.g.br[k])));
    x.free_eps = ext * 1e-6f;
    return x;
}

template <bool SIMPLE>
static __device__ __forceinline__ void mcvox_begin(const McgbMcvoxConfig &c, const McgbBuffers &b,
                                                   const MvCtx &x, MvPacket &s, Rng &rng, uint64_t p,
                                                   f3 prev_pos) {
    s.p = p;
    s.opl = 0.0f;
    s.trace_count = 0;
    s.steps = 0;
    s.events = MCGB_EV_LAUNCH;
    mcvox_launch<SIMPLE>(c, x.g, x.M, x.vox, x.lut, rng, s.pos, s.dir, s.w, s.vi, s.mat,
                         b.accumulator, prev_pos);
    s.k = MCGB_FAST_MATH ? mv_cube_k(x, s.vi) : 0;
    s.free = MCGB_FAST_MATH ? mv_ball(x, s.k) : 0.0f;
    s.pend = -1.0f;
    if (x.use_trace && (c.trace.flags & MCGB_TRACE_START))
        trace_event(c.trace, s.p, s.trace_count, s.events, s.pos, s.dir, s.w, s.opl, b.float_buffer);
}

static __device__ __forceinline__ void mcvox_end(const McgbMcvoxConfig &c, const McgbBuffers &b,
                                                 const MvCtx &x, const MvPacket &s) {
    if (x.use_trace) b.int_buffer[c.trace.count_offset + s.p] = (int32_t)s.trace_count;
}

/* One step of McKernel (mcvox), xopto/mcvox/kernel/mcvox.template.c:760-1038.

   FAST math adds free flight (albedo weight and albedo rejection).  A packet
   keeps the centre vi and half width k of a cube of voxels that all hold its
   material (the radius table; k = 0 is the packet's own voxel), and s.free,
   the radius of a ball around it inside that cube.  A sampled free path
   shorter than s.free is taken in one move without computing walls, the
   packet interacts there and s.free shrinks by the path.  A longer path
   first moves the packet through the ball to its surface and continues with
   the remainder of the path; that step intersects the walls of the cube
   rather than of one voxel.  An interaction inside the cube sets s.free to
   the distance to the cube's faces.  At a face, the voxel inside the face
   takes the place of vi and the reference's boundary logic follows; the
   voxel the packet then lies in gives the next cube.  The reference stops at
   every voxel wall and draws a new path when the next voxel holds the same
   material; the exponential free path is memoryless (the remainder of a
   path known to exceed a distance is again exponential), so the interaction
   points have the same distribution.  With a finite rmax, cubes lie inside
   the rmax sphere, so the packets end at the same steps as the reference's. */
template <int METHOD>
static __device__ __forceinline__ float mcvox_sample(const MvCtx &x, MvPacket &s, Rng &rng) {
    const float4 g0 = x.M[s.mat].g0;   /* mus, mua, step factor, mua_inv_mut */
    ++s.steps;
    float u = rng.next();
    float step = (METHOD == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT) ? mc_div(-mc_log(u), g0.x)
                                                                   : sample_step(u, g0.z);
    return fminf(step, FLT_MAX);
}

/* The rest of a step after its free path is drawn (mcvox_sample).  RMAX =
   false compiles out the rmax test (the launcher takes the SIMPLE kernels
   only without rmax). */
template <int PF, int METHOD, bool FLU, bool XTRA, bool RMAX = true>
static __device__ __forceinline__ bool mcvox_move(const McgbMcvoxConfig &c, const McgbBuffers &b,
                                                  const MvCtx &x, MvPacket &s, Rng &rng,
                                                  FluenceCache &fcache, uint32_t &status, float step) {
    constexpr bool FREE = MCGB_FAST_MATH && METHOD != MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT;
    const MvMaterial *M = x.M;
    const MvGeom &g = x.g;
    const McgbRunOptions &o = c.opt;
    uint64_t *accu = b.accumulator;
    const float4 g0 = M[s.mat].g0;   /* mus, mua, step factor, mua_inv_mut */
    const bool flight = FREE && step < s.free;
    if (FREE && !flight && s.free > 0.0f) {
        /* The path reaches beyond the ball: move through it without an
           interaction and go on with the remainder, which is again
           exponential; the reference's walk then continues from there. */
        s.pos.x = s.pos.x + s.free * s.dir.x;
        s.pos.y = s.pos.y + s.free * s.dir.y;
        s.pos.z = s.pos.z + s.free * s.dir.z;
        if (XTRA && x.track_opl) s.opl += M[s.mat].g1.x * s.free;
        step -= s.free;
        s.free = 0.0f;
    }
    f3 dist;
    float d;
    if (flight) {
        d = __int_as_float(0x7f800000);
        dist = f3{d, d, d};
    } else if (FREE) {
        /* the walls of the packet's cube (its voxel's walls when k = 0) */
        const int k = s.k;
        dist.x = g.tl[0] + (float)(s.dir.x >= 0.0f ? s.vi.x + k + 1 : s.vi.x - k) * g.vs[0] - s.pos.x;
        dist.y = g.tl[1] + (float)(s.dir.y >= 0.0f ? s.vi.y + k + 1 : s.vi.y - k) * g.vs[1] - s.pos.y;
        dist.z = g.tl[2] + (float)(s.dir.z >= 0.0f ? s.vi.z + k + 1 : s.vi.z - k) * g.vs[2] - s.pos.z;
        dist.x = (s.dir.x != 0.0f) ? mc_div(dist.x, s.dir.x) : __int_as_float(0x7f800000);
        dist.y = (s.dir.y != 0.0f) ? mc_div(dist.y, s.dir.y) : __int_as_float(0x7f800000);
        dist.z = (s.dir.z != 0.0f) ? mc_div(dist.z, s.dir.z) : __int_as_float(0x7f800000);
        d = fminf(dist.x, fminf(dist.y, dist.z));
    } else {
        /* mcsim_intersect, mcvox.template.c:173-196 */
        dist.x = g.tl[0] + (float)((s.dir.x >= 0.0f) + s.vi.x) * g.vs[0] - s.pos.x;
        dist.y = g.tl[1] + (float)((s.dir.y >= 0.0f) + s.vi.y) * g.vs[1] - s.pos.y;
        dist.z = g.tl[2] + (float)((s.dir.z >= 0.0f) + s.vi.z) * g.vs[2] - s.pos.z;
        dist.x = (s.dir.x != 0.0f) ? mc_div(dist.x, s.dir.x) : __int_as_float(0x7f800000);
        dist.y = (s.dir.y != 0.0f) ? mc_div(dist.y, s.dir.y) : __int_as_float(0x7f800000);
        dist.z = (s.dir.z != 0.0f) ? mc_div(dist.z, s.dir.z) : __int_as_float(0x7f800000);
        d = fminf(dist.x, fminf(dist.y, dist.z));
    }
    float d_ok = fminf(d, step);
    s.pos.x = s.pos.x + d_ok * s.dir.x;
    s.pos.y = s.pos.y + d_ok * s.dir.y;
    s.pos.z = s.pos.z + d_ok * s.dir.z;
    if (XTRA && x.track_opl) s.opl += M[s.mat].g1.x * d_ok;

    bool done = false;
    if (METHOD == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT) {
        float mua = g0.y;
        float fraction = 1.0f - mc_exp(-mua * d_ok);
        float deposit = fraction * s.w;
        s.w -= deposit;
        if (XTRA) s.events |= MCGB_EV_ABSORPTION;
        if (FLU) {
            float step_back = (mua != 0.0f)
                                  ? d_ok - mc_div(-mc_log(1.0f - rng.next() * fraction), mua)
                                  : 0.0f;
            f3 dp{s.pos.x - step_back * s.dir.x, s.pos.y - step_back * s.dir.y,
                  s.pos.z - step_back * s.dir.z};
            fluence_deposit<XTRA>(c.fluence, dp, deposit, mua, fcache);
        }
        if (d < step) {
            s.events |= mv_boundary(g, M, x.vox, s.dir, s.vi, s.mat, dist, rng) | MCGB_EV_BOUNDARY_HIT;
            if (!mv_valid(g, s.vi)) {
                if (s.vi.z < 0) detector_deposit<XTRA>(c.top, s.pos, s.dir, s.w, s.opl, accu, x.lut);
                else if (s.vi.z >= g.sh[2]) detector_deposit<XTRA>(c.bottom, s.pos, s.dir, s.w, s.opl, accu, x.lut);
                done = true;
            }
        } else {
            const MvMaterial &cm = M[s.mat];
            float az, ct = pf_sample<PF>(cm.pf0, cm.pf1, x.lut, rng, &az, s.dir);
            scatter_direction(s.dir, ct, az);
            if (XTRA) s.events |= MCGB_EV_SCATTERING;
        }
        if (s.w < o.packet_weight_min) {
            if (o.use_lottery) {
                if (rng.next() > o.lottery_chance) done = true;
                else s.w = mc_div(s.w, o.lottery_chance);
            } else {
                done = true;
            }
        }
    } else if (d < step) {
        if (FREE && s.k > 0) {
            /* at a face of the cube: the voxel inside that face (the
               crossing axis as mv_boundary picks it, the other axes from the
               position, kept inside the cube) */
            const int k = s.k;
            i3 f = mv_index(g, s.pos);
            f.x = clip_i(f.x, s.vi.x - k, s.vi.x + k);
            f.y = clip_i(f.y, s.vi.y - k, s.vi.y + k);
            f.z = clip_i(f.z, s.vi.z - k, s.vi.z + k);
            if (dist.x <= dist.y && dist.x <= dist.z) f.x = s.dir.x < 0.0f ? s.vi.x - k : s.vi.x + k;
            else if (dist.y <= dist.z) f.y = s.dir.y < 0.0f ? s.vi.y - k : s.vi.y + k;
            else f.z = s.dir.z < 0.0f ? s.vi.z - k : s.vi.z + k;
            s.vi = f;
        }
        uint32_t ev = mv_boundary(g, M, x.vox, s.dir, s.vi, s.mat, dist, rng);
        s.events |= ev | MCGB_EV_BOUNDARY_HIT;
        if (!mv_valid(g, s.vi)) {
            if (s.vi.z < 0) detector_deposit<XTRA>(c.top, s.pos, s.dir, s.w, s.opl, accu, x.lut);
            else if (s.vi.z >= g.sh[2]) detector_deposit<XTRA>(c.bottom, s.pos, s.dir, s.w, s.opl, accu, x.lut);
            done = true;
        } else if (FREE) {
            /* the packet's new voxel, refracted into or reflected back to */
            s.k = mv_cube_k(x, s.vi);
            s.free = mv_ball(x, s.k);
        }
    } else if (METHOD == MCGB_METHOD_ALBEDO_REJECTION) {
        if (rng.next() < g0.w) {
            float deposit = s.w;
            s.w -= deposit;
            if (XTRA) s.events |= MCGB_EV_ABSORPTION;
            done = true;
            if (FLU) fluence_deposit<XTRA>(c.fluence, s.pos, deposit, g0.y, fcache);
        } else {
            const MvMaterial &cm = M[s.mat];
            float az, ct = pf_sample<PF>(cm.pf0, cm.pf1, x.lut, rng, &az, s.dir);
            scatter_direction(s.dir, ct, az);
            if (XTRA) s.events |= MCGB_EV_SCATTERING;
        }
        if (FREE) s.free = flight ? s.free - step : mv_clearance(x, s.vi, s.k, s.pos);
    } else {
        float deposit = s.w * g0.w;
        s.w -= deposit;
        if (XTRA) s.events |= MCGB_EV_ABSORPTION;
        if (FLU) fluence_deposit<XTRA>(c.fluence, s.pos, deposit, g0.y, fcache);
        const MvMaterial &cm = M[s.mat];
        float az, ct = pf_sample<PF>(cm.pf0, cm.pf1, x.lut, rng, &az, s.dir);
        scatter_direction(s.dir, ct, az);
        if (XTRA) s.events |= MCGB_EV_SCATTERING;
        if (s.w < o.packet_weight_min) {
            if (o.use_lottery) {
                if (rng.next() > o.lottery_chance) done = true;
                else s.w = mc_div(s.w, o.lottery_chance);
            } else {
                done = true;
            }
        }
        if (FREE) s.free = flight ? s.free - step : mv_clearance(x, s.vi, s.k, s.pos);
    }
    /* mcvox.template.c:1004-1008 */
    bool escaped = s.w <= 0.0f;
    if (RMAX && x.use_rmax) {
        f3 dd{s.pos.x - x.src_pos.x, s.pos.y - x.src_pos.y, s.pos.z - x.src_pos.z};
        escaped = escaped || dot3(dd, dd) > x.rmax2;
    }
    if (escaped) {
        done = true;
        if (XTRA) s.events |= MCGB_EV_ESCAPED;
    }
    if (XTRA && x.use_trace) {
        if (done) s.events |= MCGB_EV_TERMINATED;
        if (c.trace.flags == MCGB_TRACE_ALL || ((c.trace.flags & MCGB_TRACE_END) && done))
            trace_event(c.trace, s.p, s.trace_count, s.events, s.pos, s.dir, s.w, s.opl, b.float_buffer);
        s.events = 0;
    }
    if (XTRA && !done && s.steps >= x.max_steps) {
        done = true;
        status |= MCGB_STATUS_STEP_LIMIT;
    }
    return done;
}

template <int PF, int METHOD, bool FLU, bool XTRA, bool RMAX = true>
static __device__ __forceinline__ bool mcvox_step(const McgbMcvoxConfig &c, const McgbBuffers &b,
                                                  const MvCtx &x, MvPacket &s, Rng &rng,
                                                  FluenceCache &fcache, uint32_t &status) {
    const float step = mcvox_sample<METHOD>(x, s, rng);
    return mcvox_move<PF, METHOD, FLU, XTRA, RMAX>(c, b, x, s, rng, fcache, status, step);
}

template <int PF>
static __device__ __forceinline__ const float *mcvox_stage(const McgbMcvoxConfig &c, const McgbBuffers &b,
                                                           MvSmem &sm, float *s_lut, int lut_in_smem) {
    for (uint32_t i = threadIdx.x; i < c.num_materials; i += blockDim.x) {
        const McgbMaterial &m = b.materials[i];
        MvMaterial h;
        h.g0 = make_float4(m.mus, m.mua, step_factor(m.inv_mut), m.mua_inv_mut);
        h.g1 = make_float4(m.n, 0.0f, 0.0f, 0.0f);
        pf_prepare(PF, m.pf, h.pf0, h.pf1);
        sm.materials[i] = h;
    }
    if (lut_in_smem)
        for (uint64_t i = threadIdx.x; i < b.fp_lut_size; i += blockDim.x) s_lut[i] = b.fp_lut[i];
    __syncthreads();
    return lut_in_smem ? s_lut : b.fp_lut;
}

static __device__ __forceinline__ void mv_finish(const McgbBuffers &b, uint64_t steps, uint64_t packets,
                                                 uint32_t status, bool count_thread) {
    atomicAdd((unsigned long long *)(b.counters + MCGB_CNT_STEPS), (unsigned long long)steps);
    atomicAdd((unsigned long long *)(b.counters + MCGB_CNT_PACKETS), (unsigned long long)packets);
    if (count_thread) atomicAdd((unsigned long long *)(b.counters + MCGB_CNT_THREADS), 1ull);
    if (status) atomicOr((unsigned long long *)(b.counters + MCGB_CNT_STATUS), (unsigned long long)status);
}

/* STATIC scheduling (thread t owns stream t). */
template <int PF, int METHOD, bool FLU>
__global__ void __launch_bounds__(256)
mcvox_transport_kernel(const __grid_constant__ McgbMcvoxConfig c, const McgbBuffers b,
                       uint64_t deadline_ns, int lut_in_smem, uint32_t packets_per_item) {
    __shared__ MvSmem sm;
    extern __shared__ float s_lut[];
    const float *lut = mcvox_stage<PF>(c, b, sm, s_lut, lut_in_smem);
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c.num_streams || t >= c.num_packets) return;
    const uint64_t t_deadline = globaltimer_ns() + deadline_ns;
    const MvCtx x = mcvox_ctx(c, b, sm.materials, lut);
    const uint64_t T = c.num_streams;
    Rng rng{b.rng_x[t], b.rng_a[t]};
    FluenceCache fcache = fluence_cache(c.fluence, b.accumulator);
    uint64_t steps = 0, packets = 0;
    uint32_t iter = 0, status = 0;
    MvPacket s;
    s.pos = f3{0.0f, 0.0f, 0.0f};
    mcvox_begin<false>(c, b, x, s, rng, t, s.pos);
    for (;;) {
        if (mcvox_step<PF, METHOD, FLU, true>(c, b, x, s, rng, fcache, status)) {
            ++packets;
            steps += s.steps;
            mcvox_end(c, b, x, s);
            uint64_t p = s.p + T;
            if (p >= c.num_packets) {
                s.steps = 0;
                break;
            }
            mcvox_begin<false>(c, b, x, s, rng, p, s.pos);
        }
        if (((++iter) & 1023u) == 0) {
            if (globaltimer_ns() > t_deadline) { status |= MCGB_STATUS_TIMEOUT; break; }
            if (*(volatile uint64_t *)(b.counters + MCGB_CNT_ABORT)) { status |= MCGB_STATUS_ABORTED; break; }
        }
    }
    steps += s.steps;
    if (FLU) fcache.flush();
    b.rng_x[t] = rng.x;
    mv_finish(b, steps, packets, status, true);
}

/* DYNAMIC scheduling (per-packet streams, warp refill). */
template <int PF, int METHOD, bool FLU, bool XTRA, bool SIMPLE>
__global__ void __launch_bounds__(128)
mcvox_dynamic_kernel(const __grid_constant__ McgbMcvoxConfig c, const McgbBuffers b,
                     uint64_t deadline_ns, int lut_in_smem, uint32_t packets_per_item) {
    __shared__ MvSmem sm;
    extern __shared__ float s_lut[];
    const float *lut = mcvox_stage<PF>(c, b, sm, s_lut, lut_in_smem);
    /* the phased loop: FAST free flight in the plain kernels */
    constexpr bool PHASED = MCGB_FAST_MATH && METHOD != MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT && !XTRA;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t t_deadline = globaltimer_ns() + deadline_ns;
    const MvCtx x = mcvox_ctx(c, b, sm.materials, lut);
    const uint64_t N = c.num_packets;
    const uint64_t B = packets_per_item;
    unsigned long long *queue = (unsigned long long *)(b.counters + MCGB_CNT_QUEUE);
    uint64_t item_next = 0, item_end = 0;
    bool more = true, active = false;
    Rng rng{0ull, 1u};
    FluenceCache fcache = fluence_cache(c.fluence, b.accumulator);
    uint64_t steps = 0, packets = 0;
    uint32_t iter = 0, status = 0;
    MvPacket s;
    s.steps = 0;
    for (;;) {
        uint32_t need = __ballot_sync(0xffffffffu, !active);
        while (need && more) {
            if (item_next >= item_end) {
                unsigned long long item = 0;
                if (lane == 0) item = atomicAdd(queue, 1ull);
                item = __shfl_sync(0xffffffffu, item, 0);
                item_next = (uint64_t)item * B;
                if (item_next >= N) {
                    more = false;
                    break;
                }
                item_end = min(item_next + B, N);
            }
            uint32_t avail = (uint32_t)min(item_end - item_next, (uint64_t)32);
            uint32_t rank = __popc(need & ((1u << lane) - 1u));
            bool mine = ((need >> lane) & 1u) && rank < avail;
            if (mine) {
                uint64_t p = item_next + rank;
                uint64_t xs;
                uint32_t as;
                br_packet_stream(c.opt.seed, 0u, c.opt.packet_offset + p, b.rng_a, c.num_streams, &xs, &as);
                rng = Rng{xs, as};
                mcvox_begin<SIMPLE>(c, b, x, s, rng, p, f3{0.0f, 0.0f, 0.0f});
                active = true;
            }
            uint32_t taken = __ballot_sync(0xffffffffu, mine);
            item_next += __popc(taken);
            need &= ~taken;
        }
        if (!__any_sync(0xffffffffu, active)) break;
        /* 32 steps between refills (+0.6 % against 16 on the skin and
           vessel grid); the step body is not unrolled (two bodies per
           iteration cost 10 % here) */
#pragma unroll 1
        for (int k = 0; k < 32; ++k) {
            if (PHASED) {
                /* Phased steps: every lane draws its path; lanes whose path
                   leaves their ball (wall steps) wait until they are at
                   least half of the active lanes, so that the wall code
                   runs for many lanes at once while the others fly.  A
                   lane's own sequence of operations is that of mcvox_step. */
                if (active && s.pend < 0.0f) s.pend = mcvox_sample<METHOD>(x, s, rng);
                const bool wall = active && !(s.pend < s.free);
                const uint32_t act_m = __ballot_sync(0xffffffffu, active);
                const uint32_t wall_m = __ballot_sync(0xffffffffu, wall);
                const bool run_walls = 2 * __popc(wall_m) >= __popc(act_m);
                if (active && (run_walls || !wall)) {
                    const float step = s.pend;
                    s.pend = -1.0f;
                    if (mcvox_move<PF, METHOD, FLU, XTRA, XTRA || !SIMPLE>(c, b, x, s, rng, fcache, status, step)) {
                        ++packets;
                        steps += s.steps;
                        s.steps = 0;
                        mcvox_end(c, b, x, s);
                        active = false;
                    }
                }
            } else if (active && mcvox_step<PF, METHOD, FLU, XTRA, XTRA || !SIMPLE>(c, b, x, s, rng, fcache, status)) {
                ++packets;
                steps += s.steps;
                s.steps = 0;
                mcvox_end(c, b, x, s);
                active = false;
            }
        }
        iter += 32;
        if ((iter & 1023u) == 0) {
            uint32_t stop = 0;
            if (lane == 0) {
                if (globaltimer_ns() > t_deadline) stop = MCGB_STATUS_TIMEOUT;
                else if (*(volatile uint64_t *)(b.counters + MCGB_CNT_ABORT)) stop = MCGB_STATUS_ABORTED;
            }
            stop = __shfl_sync(0xffffffffu, stop, 0);
            if (stop) {
                status |= stop;
                break;
            }
        }
    }
    steps += s.steps;
    if (FLU) fcache.flush();
    mv_finish(b, steps, packets, status, packets > 0);
}

}  // namespace MCGB_NS
