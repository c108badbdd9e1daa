// Grid-side kernels: Becke partition weights and AO evaluation.
#include <cstdio>

#include "common.h"
#include "kernels.h"

namespace cgb {

namespace {

constexpr int kNcart = (kMaxL + 1) * (kMaxL + 2) / 2;
__constant__ double c_sh[kMaxL + 1][2 * kMaxL + 1][kNcart];

// GridGeneration.cpp:50-71 with the point-to-atom distances precomputed.
__device__ __forceinline__ double becke_s(double rb, double rc, double rbc) {
    const double mu = (rb - rc) / rbc;
    const double p1 = 1.5 * mu - 0.5 * mu * mu * mu;
    const double p2 = 1.5 * p1 - 0.5 * p1 * p1 * p1;
    const double p3 = 1.5 * p2 - 0.5 * p2 * p2 * p2;
    return 0.5 * (1 - p3);
}

// One thread per point.  Shared memory: atom coordinates, atom-atom
// distances and this CTA's point-atom distances (natoms <= kBeckeSmemAtoms).
constexpr int kBeckeThreads = 128;
constexpr int kBeckeSmemAtoms = 64;

__global__ void __launch_bounds__(kBeckeThreads) becke_kernel(int natoms, const double* __restrict__ atoms, long npts,
                                                              const double* __restrict__ px, const double* __restrict__ py,
                                                              const double* __restrict__ pz, const int* __restrict__ owner,
                                                              const double* __restrict__ w_in, double* __restrict__ w_out) {
    extern __shared__ double sm[];
    double* Rab = sm;                                  // natoms^2
    double* dist = sm + natoms * natoms;               // natoms x kBeckeThreads
    for (int i = threadIdx.x; i < natoms * natoms; i += blockDim.x) {
        const int a = i / natoms, b = i % natoms;
        const double dx = atoms[3 * a] - atoms[3 * b], dy = atoms[3 * a + 1] - atoms[3 * b + 1],
                     dz = atoms[3 * a + 2] - atoms[3 * b + 2];
        Rab[i] = sqrt(dx * dx + dy * dy + dz * dz);
    }
    __syncthreads();
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npts) return;
    const double x = px[k], y = py[k], z = pz[k];
    for (int a = 0; a < natoms; a++) {
        const double dx = x - atoms[3 * a], dy = y - atoms[3 * a + 1], dz = z - atoms[3 * a + 2];
        dist[a * kBeckeThreads + threadIdx.x] = sqrt(dx * dx + dy * dy + dz * dz);
    }
    const int own = owner[k];
    double total = 0, mine = 0;
    for (int b = 0; b < natoms; b++) {
        const double rb = dist[b * kBeckeThreads + threadIdx.x];
        double pb = 1;
        for (int c = 0; c < natoms; c++) {
            if (c == b) continue;
            pb *= becke_s(rb, dist[c * kBeckeThreads + threadIdx.x], Rab[b * natoms + c]);
        }
        total += pb;
        if (b == own) mine = pb;
    }
    w_out[k] = w_in[k] * (mine / total);
}

// Same without shared-memory caches, for large atom counts.
__global__ void becke_kernel_big(int natoms, const double* __restrict__ atoms, long npts, const double* __restrict__ px,
                                 const double* __restrict__ py, const double* __restrict__ pz,
                                 const int* __restrict__ owner, const double* __restrict__ w_in,
                                 double* __restrict__ w_out) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npts) return;
    const double x = px[k], y = py[k], z = pz[k];
    const int own = owner[k];
    double total = 0, mine = 0;
    for (int b = 0; b < natoms; b++) {
        const double bx = atoms[3 * b], by = atoms[3 * b + 1], bz = atoms[3 * b + 2];
        const double rb = sqrt((x - bx) * (x - bx) + (y - by) * (y - by) + (z - bz) * (z - bz));
        double pb = 1;
        for (int c = 0; c < natoms; c++) {
            if (c == b) continue;
            const double cx = atoms[3 * c], cy = atoms[3 * c + 1], cz = atoms[3 * c + 2];
            const double rc = sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy) + (z - cz) * (z - cz));
            const double rbc = sqrt((bx - cx) * (bx - cx) + (by - cy) * (by - cy) + (bz - cz) * (bz - cz));
            pb *= becke_s(rb, rc, rbc);
        }
        total += pb;
        if (b == own) mine = pb;
    }
    w_out[k] = w_in[k] * (mine / total);
}

// One CTA per grid block, one thread per (padded) point; loops over the
// block's screened shells.  ao layout: [comp][n_b][ng] from blocks[b].ao_off.
__global__ void __launch_bounds__(kMaxBlockPts) ao_kernel(const BlockDesc* __restrict__ blocks,
                                                          const int* __restrict__ block_shells, DevShells sh,
                                                          const double* __restrict__ px, const double* __restrict__ py,
                                                          const double* __restrict__ pz, int ncomp,
                                                          double* __restrict__ ao) {
    const BlockDesc bd = blocks[blockIdx.x];
    const int g = threadIdx.x;
    if (g >= bd.ng) return;
    const double X = px[bd.pt_off + g], Y = py[bd.pt_off + g], Z = pz[bd.pt_off + g];
    double* out = ao + bd.ao_off;
    const long comp_stride = (long)bd.nb * bd.ng;
    int mu = 0;
    for (int is = 0; is < bd.nsh; is++) {
        const int s = block_shells[bd.sh_off + is];
        const int l = sh.l[s], type = sh.type[s], np = sh.nprim[s], po = sh.prim_off[s];
        const double x = X - sh.xyz[3 * s], y = Y - sh.xyz[3 * s + 1], z = Z - sh.xyz[3 * s + 2];
        const double r2 = x * x + y * y + z * z;
        double t0 = 0, t1 = 0, t2 = 0;
        for (int p = 0; p < np; p++) {  // GridAO.cpp:113-124
            const double e = sh.exps[po + p];
            const double t = sh.coefs[po + p] * exp(-e * r2);
            t0 += t;
            t1 += t * e;
            t2 += t * e * e;
        }
        const double A = t0, Ax = -2 * x * t1, Ay = -2 * y * t1, Az = -2 * z * t1;
        // second derivatives of the radial part: d_t d_r R = 4 x_t x_r t2 - 2 delta_tr t1
        const double Axx = 4 * x * x * t2 - 2 * t1, Ayy = 4 * y * y * t2 - 2 * t1, Azz = 4 * z * z * t2 - 2 * t1;
        const double Axy = 4 * x * y * t2, Axz = 4 * x * z * t2, Ayz = 4 * y * z * t2;
        double xp[kMaxL + 1], yp[kMaxL + 1], zp[kMaxL + 1];
        xp[0] = yp[0] = zp[0] = 1;
        for (int i = 1; i <= l; i++) {
            xp[i] = xp[i - 1] * x;
            yp[i] = yp[i - 1] * y;
            zp[i] = zp[i - 1] * z;
        }
        const int nf = 2 * l + 1;
        for (int f = 0; f < nf; f++) {
            // Cartesian P shells (type 1) are x, y, z = table rows m = +1, -1, 0.
            const int row = (type == 1) ? (f == 0 ? 2 : f - 1) : f;
            double Q = 0, Qx = 0, Qy = 0, Qz = 0;
            double Qxx = 0, Qxy = 0, Qxz = 0, Qyy = 0, Qyz = 0, Qzz = 0;
            int k = 0;
            for (int a = l; a >= 0; a--)
                for (int b = l - a; b >= 0; b--, k++) {
                    const double c = c_sh[l][row][k];
                    if (c == 0) continue;
                    const int cc = l - a - b;
                    Q += c * xp[a] * yp[b] * zp[cc];
                    if (ncomp > 1) {
                        if (a) Qx += c * a * xp[a - 1] * yp[b] * zp[cc];
                        if (b) Qy += c * b * xp[a] * yp[b - 1] * zp[cc];
                        if (cc) Qz += c * cc * xp[a] * yp[b] * zp[cc - 1];
                    }
                    if (ncomp > 4) {  // Hessian of the angular polynomial
                        if (a > 1) Qxx += c * a * (a - 1) * xp[a - 2] * yp[b] * zp[cc];
                        if (b > 1) Qyy += c * b * (b - 1) * xp[a] * yp[b - 2] * zp[cc];
                        if (cc > 1) Qzz += c * cc * (cc - 1) * xp[a] * yp[b] * zp[cc - 2];
                        if (a && b) Qxy += c * a * b * xp[a - 1] * yp[b - 1] * zp[cc];
                        if (a && cc) Qxz += c * a * cc * xp[a - 1] * yp[b] * zp[cc - 1];
                        if (b && cc) Qyz += c * b * cc * xp[a] * yp[b - 1] * zp[cc - 1];
                    }
                }
            const long o = (long)(mu + f) * bd.ng + g;
            out[o] = A * Q;  // GridAO.cpp:180-184 (product rule)
            if (ncomp > 1) {
                out[comp_stride + o] = Ax * Q + A * Qx;
                out[2 * comp_stride + o] = Ay * Q + A * Qy;
                out[3 * comp_stride + o] = Az * Q + A * Qz;
            }
            if (ncomp > 4) {  // xx, xy, xz, yy, yz, zz: d_t d_r (R Q)
                out[4 * comp_stride + o] = Axx * Q + 2 * Ax * Qx + A * Qxx;
                out[5 * comp_stride + o] = Axy * Q + Ax * Qy + Ay * Qx + A * Qxy;
                out[6 * comp_stride + o] = Axz * Q + Ax * Qz + Az * Qx + A * Qxz;
                out[7 * comp_stride + o] = Ayy * Q + 2 * Ay * Qy + A * Qyy;
                out[8 * comp_stride + o] = Ayz * Q + Ay * Qz + Az * Qy + A * Qyz;
                out[9 * comp_stride + o] = Azz * Q + 2 * Az * Qz + A * Qzz;
            }
        }
        mu += nf;
    }
}

}  // namespace

void upload_solid_harmonics() {
    static double table[kMaxL + 1][2 * kMaxL + 1][kNcart];
    solid_harmonic_table(table);
    CGB_CUDA(cudaMemcpyToSymbol(c_sh, table, sizeof(table)));
}

void launch_becke(int natoms, const double* d_atoms, long npts, const double* x, const double* y, const double* z,
                  const int* owner, const double* w_in, double* w_out, cudaStream_t s) {
    if (npts == 0) return;
    const unsigned grid = (unsigned)((npts + kBeckeThreads - 1) / kBeckeThreads);
    if (natoms <= kBeckeSmemAtoms) {
        const size_t smem = sizeof(double) * ((size_t)natoms * natoms + (size_t)natoms * kBeckeThreads);
        CGB_CUDA(cudaFuncSetAttribute(becke_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        becke_kernel<<<grid, kBeckeThreads, smem, s>>>(natoms, d_atoms, npts, x, y, z, owner, w_in, w_out);
    } else {
        becke_kernel_big<<<grid, kBeckeThreads, 0, s>>>(natoms, d_atoms, npts, x, y, z, owner, w_in, w_out);
    }
    CGB_CUDA(cudaGetLastError());
}

void launch_ao(int nblocks, const BlockDesc* d_blocks, const int* d_block_shells, DevShells sh, const double* x,
               const double* y, const double* z, int ncomp, double* ao, cudaStream_t s) {
    if (nblocks == 0) return;
    ao_kernel<<<nblocks, kMaxBlockPts, 0, s>>>(d_blocks, d_block_shells, sh, x, y, z, ncomp, ao);
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
