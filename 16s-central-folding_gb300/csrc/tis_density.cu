// Ion density grids on the device (the reference's analysis/Mg_distribution_3D/
// calc_Mg_density.py, which histograms Mg positions read back from DCD frames
// fitted by bestfit_motifs.py): per frame, an optional least-squares superposition
// of selected beads onto reference coordinates, then every ion of one kind binned
// into a 3-D grid, all on the handle's stream with no host synchronisation.
#include "tis_kernels.cuh"

namespace tis {
namespace {

constexpr int kFitThreads = 256;

// Largest-eigenvalue eigenvector of the symmetric 4x4 matrix a (cyclic Jacobi
// rotations, at most 50 sweeps).
__device__ void eig4_max(double a[4][4], double q[4])
{
    double v[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < 4; ++i)
            for (int j = i + 1; j < 4; ++j) off += a[i][j] * a[i][j];
        if (off < 1e-300) break;
        for (int p = 0; p < 4; ++p)
            for (int r = p + 1; r < 4; ++r) {
                if (a[p][r] == 0.0) continue;
                const double th = 0.5 * (a[r][r] - a[p][p]) / a[p][r];
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 4; ++k) {  // a <- J^T a J
                    const double akp = a[k][p], akr = a[k][r];
                    a[k][p] = c * akp - s * akr;
                    a[k][r] = s * akp + c * akr;
                }
                for (int k = 0; k < 4; ++k) {
                    const double apk = a[p][k], ark = a[r][k];
                    a[p][k] = c * apk - s * ark;
                    a[r][k] = s * apk + c * ark;
                }
                for (int k = 0; k < 4; ++k) {
                    const double vkp = v[k][p], vkr = v[k][r];
                    v[k][p] = c * vkp - s * vkr;
                    v[k][r] = s * vkp + c * vkr;
                }
            }
    }
    int best = 0;
    for (int i = 1; i < 4; ++i)
        if (a[i][i] > a[best][best]) best = i;
    for (int k = 0; k < 4; ++k) q[k] = v[k][best];
}

// One block: centroids and the correlation of the fit beads with their reference
// positions, then (thread 0) the rotation of Horn's quaternion method (J. Opt.
// Soc. Am. A 4, 629 (1987)) taking the frame onto the reference:
// out = {R (9, row-major), frame centroid (3), reference centroid (3), rmsd}.
__global__ void __launch_bounds__(kFitThreads) k_fit(Dev d, int r, int n_fit, const int *idx, const double *ref,
                                                     double *out)
{
    __shared__ double s_red[15][kFitThreads / 32];
    const RepParams *R = d.rp + r;
    double acc[15] = {0};  // sx sy sz, ry rx.. (3), sum x_a y_b (9)
    for (int i = threadIdx.x; i < n_fit; i += blockDim.x) {
        const int p = R->p0 + idx[i];
        const double x[3] = {d.x[p], d.y[p], d.z[p]}, y[3] = {ref[3 * i], ref[3 * i + 1], ref[3 * i + 2]};
        for (int a = 0; a < 3; ++a) {
            acc[a] += x[a];
            acc[3 + a] += y[a];
            for (int b = 0; b < 3; ++b) acc[6 + 3 * a + b] += x[a] * y[b];
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 15; ++k) {
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
        if (lane == 0) s_red[k][warp] = acc[k];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double t[15];
    for (int k = 0; k < 15; ++k) {
        t[k] = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t[k] += s_red[k][w];
    }
    const double inv = 1.0 / n_fit;
    const double xc[3] = {t[0] * inv, t[1] * inv, t[2] * inv}, yc[3] = {t[3] * inv, t[4] * inv, t[5] * inv};
    double S[3][3];  // sum (x - xc)_a (y - yc)_b
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) S[a][b] = t[6 + 3 * a + b] - n_fit * xc[a] * yc[b];
    double N[4][4] = {
        {S[0][0] + S[1][1] + S[2][2], S[1][2] - S[2][1], S[2][0] - S[0][2], S[0][1] - S[1][0]},
        {S[1][2] - S[2][1], S[0][0] - S[1][1] - S[2][2], S[0][1] + S[1][0], S[2][0] + S[0][2]},
        {S[2][0] - S[0][2], S[0][1] + S[1][0], -S[0][0] + S[1][1] - S[2][2], S[1][2] + S[2][1]},
        {S[0][1] - S[1][0], S[2][0] + S[0][2], S[1][2] + S[2][1], -S[0][0] - S[1][1] + S[2][2]}};
    double q[4];
    eig4_max(N, q);
    const double q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
    const double Rm[9] = {q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3, 2 * (q1 * q2 - q0 * q3), 2 * (q1 * q3 + q0 * q2),
                          2 * (q1 * q2 + q0 * q3), q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3, 2 * (q2 * q3 - q0 * q1),
                          2 * (q1 * q3 - q0 * q2), 2 * (q2 * q3 + q0 * q1), q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3};
    for (int k = 0; k < 9; ++k) out[k] = Rm[k];
    for (int a = 0; a < 3; ++a) {
        out[9 + a] = xc[a];
        out[12 + a] = yc[a];
    }
    double e2 = 0.0;  // rmsd after the fit, from the beads themselves
    for (int i = 0; i < n_fit; ++i) {
        const int p = R->p0 + idx[i];
        const double x[3] = {d.x[p] - xc[0], d.y[p] - xc[1], d.z[p] - xc[2]};
        for (int a = 0; a < 3; ++a) {
            const double v = Rm[3 * a] * x[0] + Rm[3 * a + 1] * x[1] + Rm[3 * a + 2] * x[2] + yc[a] - ref[3 * i + a];
            e2 += v * v;
        }
    }
    out[15] = sqrt(e2 * inv);
}

// every particle of replica r of `kind`: its (fitted) position binned into the grid
// lo + delta * [0, dims); the upper faces belong to the last bins (numpy.histogramdd)
__global__ void k_density(Dev d, int r, int kind, const double *fit, double lo0, double lo1, double lo2, double delta,
                          int nx, int ny, int nz, unsigned long long *grid)
{
    const RepParams *R = d.rp + r;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R->n) return;
    const int p = R->p0 + i;
    if (((d.q[p].w >> 8) & 0xff) != kind) return;
    double x[3] = {d.x[p], d.y[p], d.z[p]};
    if (fit) {
        const double c[3] = {x[0] - fit[9], x[1] - fit[10], x[2] - fit[11]};
        for (int a = 0; a < 3; ++a) x[a] = fit[3 * a] * c[0] + fit[3 * a + 1] * c[1] + fit[3 * a + 2] * c[2] + fit[12 + a];
    }
    const double lo[3] = {lo0, lo1, lo2};
    const int dims[3] = {nx, ny, nz};
    int b[3];
    for (int a = 0; a < 3; ++a) {
        const double u = (x[a] - lo[a]) / delta;
        if (!(u >= 0.0) || u > (double)dims[a]) return;
        b[a] = min((int)floor(u), dims[a] - 1);
    }
    atomicAdd(grid + ((size_t)b[0] * ny + b[1]) * nz + b[2], 1ull);
}

}  // namespace

void launch_fit(const Dev &d, cudaStream_t s, int r, int n_fit, const int *idx, const double *ref, double *out)
{
    k_fit<<<1, kFitThreads, 0, s>>>(d, r, n_fit, idx, ref, out);
}

void launch_density(const Dev &d, cudaStream_t s, int r, int n, int kind, const double *fit, const double lo[3],
                    double delta, const int dims[3], unsigned long long *grid)
{
    k_density<<<(n + 255) / 256, 256, 0, s>>>(d, r, kind, fit, lo[0], lo[1], lo[2], delta, dims[0], dims[1], dims[2],
                                               grid);
}

}  // namespace tis
