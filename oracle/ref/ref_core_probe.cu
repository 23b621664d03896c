// ref_core_probe.cu — TEST INFRASTRUCTURE.  Compiles the reference's own
// KaminoGPU/kernel/KaminoCore.cu unchanged (included below from the
// reference tree) into a cubin, and adds two probe kernels that call the
// reference's validateCoord (KaminoCore.cu:11-29) so the harness can read its
// pole-wrap decisions directly.  Only the index lines after validateCoord
// (KaminoCore.cu:42-52 and their twins) are restated here.
#include "KaminoCore.cu"

extern "C" __global__ void kref_probe_index(int kind, const float* phiRaw, const float* thetaRaw,
                                            long long n, int* out, float* alpha)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    fReal phi, theta;
    if (kind == 0) {
        phi = phiRaw[k] - gridLenGlobal * vPhiPhiOffset;
        theta = thetaRaw[k] - gridLenGlobal * vPhiThetaOffset;
    } else if (kind == 1) {
        phi = phiRaw[k] - gridLenGlobal * vThetaPhiOffset;
        theta = thetaRaw[k] - gridLenGlobal * vThetaThetaOffset;
    } else {
        phi = phiRaw[k] - gridLenGlobal * centeredPhiOffset;
        theta = thetaRaw[k] - gridLenGlobal * centeredThetaOffset;
    }
    fReal invGridLen = 1.0 / gridLenGlobal;
    fReal isFlippedPole = validateCoord(phi, theta);
    fReal normedPhi = phi * invGridLen;
    fReal normedTheta = theta * invGridLen;
    int phiIndex = static_cast<int>(floorf(normedPhi));
    int thetaIndex = static_cast<int>(floorf(normedTheta));
    fReal alphaPhi = normedPhi - static_cast<fReal>(phiIndex);
    fReal alphaTheta = normedTheta - static_cast<fReal>(thetaIndex);
    size_t poleRow = (kind == 1) ? nThetaGlobal - 2 : nThetaGlobal - 1;
    bool pole = (thetaIndex == 0 && isFlippedPole == -1.0f) || thetaIndex == poleRow;
    out[4 * k] = (int)(phiIndex % nPhiGlobal);
    out[4 * k + 1] = thetaIndex;
    out[4 * k + 2] = isFlippedPole == -1.0f;
    out[4 * k + 3] = pole;
    alpha[2 * k] = alphaPhi;
    alpha[2 * k + 1] = alphaTheta;
}

extern "C" __global__ void kref_probe_wrap(float* phi, float* theta, long long n, int* cells)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    fReal p = phi[k], t = theta[k];
    validateCoord(p, t);
    phi[k] = p;
    theta[k] = t;
    cells[2 * k] = (int)floorf(p / gridLenGlobal);
    cells[2 * k + 1] = (int)floorf(t / gridLenGlobal);
}
