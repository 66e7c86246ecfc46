/*
 * Oracle (test infrastructure only): a plain-C restatement of the reference's
 * grid rotation, used by tests/, bench.py's CPU baseline and smoke() as the
 * checker.  Nothing in the product links or calls this file.
 *
 * Follows src/powerfit_em/_extensions.c:7-196 (rotate_grid3d):
 *   for every integer offset p = (z, y, x) with |p|^2 <= radius^2, the output
 *   voxel p (wrapped periodically into the grid) receives the input sampled at
 *   the point q = R^T p, where
 *       q_x = r0*x + r3*y + r6*z,  q_y = r1*x + r4*y + r7*z,  q_z = r2*x + r5*y + r8*z
 *   (accumulated in the order z, then y, then x, as the reference loops do).
 *   nearest != 0: input at (round(q_z), round(q_y), round(q_x)) wrapped once
 *   into the grid (C round(): halves away from zero).
 *   nearest == 0: trilinear interpolation between floor(q) and floor(q)+1 with
 *   periodic wrap.
 *   Output voxels outside the sphere are not written.  Loop order is
 *   z, y, x ascending, so when two offsets wrap onto the same voxel the later
 *   one (larger coordinate) wins, as in the reference.
 *
 * Built with -ffp-contract=off so that the coordinate sums round exactly like
 * the reference's x86-64 build (no fused multiply-add there either).
 */
#include <math.h>
#include <stdint.h>

static inline long wrap_index(long i, long n)
{
    /* Indices here lie in [-n, 2n): one add or subtract suffices. */
    if (i < 0) return i + n;
    if (i >= n) return i - n;
    return i;
}

int oracle_rotate_grid3d(const double *grid, int nz, int ny, int nx,
                         const double *rotmat, int radius, double *out,
                         int nearest)
{
    const long sx = 1, sy = nx, sz = (long)nx * ny;
    const long r2 = (long)radius * radius;
    if (nz <= 0 || ny <= 0 || nx <= 0 || radius < 0) return -1;

    for (int z = -radius; z <= radius; ++z) {
        const long dz2 = (long)z * z;
        if (dz2 > r2) continue;
        const double qx_z = rotmat[6] * z, qy_z = rotmat[7] * z, qz_z = rotmat[8] * z;
        const long oz = wrap_index(z, nz);
        for (int y = -radius; y <= radius; ++y) {
            const long dzy2 = dz2 + (long)y * y;
            if (dzy2 > r2) continue;
            const double qx_zy = qx_z + rotmat[3] * y;
            const double qy_zy = qy_z + rotmat[4] * y;
            const double qz_zy = qz_z + rotmat[5] * y;
            const long oy = wrap_index(y, ny);
            for (int x = -radius; x <= radius; ++x) {
                if (dzy2 + (long)x * x > r2) continue;
                const double qx = qx_zy + rotmat[0] * x;
                const double qy = qy_zy + rotmat[1] * x;
                const double qz = qz_zy + rotmat[2] * x;
                const long ox = wrap_index(x, nx);
                const long o = oz * sz + oy * sy + ox * sx;
                if (nearest) {
                    const long ix = wrap_index((long)round(qx), nx);
                    const long iy = wrap_index((long)round(qy), ny);
                    const long iz = wrap_index((long)round(qz), nz);
                    out[o] = grid[iz * sz + iy * sy + ix];
                } else {
                    const long x0 = (long)floor(qx), y0 = (long)floor(qy), z0 = (long)floor(qz);
                    const double fx = qx - x0, fy = qy - y0, fz = qz - z0;
                    const double gx = 1.0 - fx, gy = 1.0 - fy, gz = 1.0 - fz;
                    const long ix0 = wrap_index(x0, nx), ix1 = wrap_index(x0 + 1, nx);
                    const long iy0 = wrap_index(y0, ny) * sy, iy1 = wrap_index(y0 + 1, ny) * sy;
                    const long iz0 = wrap_index(z0, nz) * sz, iz1 = wrap_index(z0 + 1, nz) * sz;
                    /* x first, then y, then z, as in the reference */
                    const double c00 = grid[iz0 + iy0 + ix0] * gx + grid[iz0 + iy0 + ix1] * fx;
                    const double c10 = grid[iz0 + iy1 + ix0] * gx + grid[iz0 + iy1 + ix1] * fx;
                    const double c01 = grid[iz1 + iy0 + ix0] * gx + grid[iz1 + iy0 + ix1] * fx;
                    const double c11 = grid[iz1 + iy1 + ix0] * gx + grid[iz1 + iy1 + ix1] * fx;
                    const double c0 = c00 * gy + c10 * fy;
                    const double c1 = c01 * gy + c11 * fy;
                    out[o] = c0 * gz + c1 * fz;
                }
            }
        }
    }
    return 0;
}
