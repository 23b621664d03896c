// TEST INFRASTRUCTURE: the reference's own FBM curl-noise velocity
// initialiser, run on the host to make golden vectors.
//
// KaminoSolver::initialize_velocity, FBM, interpNoise2D and rand
// (KaminoGPU/kernel/KaminoInitializer.cu:3-134) are plain host C++.  That
// file and vectorUtil.cu are compiled unchanged from the reference tree
// beside this one (see oracle/build.py, build_ref_fbm); this file supplies
// what they need from the rest of the reference without CUDA: a solver
// object whose constructor only sets the members initialize_velocity reads
// (as KaminoSolver.cu:12-16, 51-54 set them), host-only KaminoQuantity
// buffers (KaminoQuantity.cu:20-27, 43-73 without the device copies) and a
// copyVelocity2GPU that copies nothing.  The reference's own constructor
// calls initialize_velocity (KaminoSolver.cu:59); here ref_fbm_velocity
// calls it and returns the host buffers it filled.
#include <cmath>
#include <cstring>
#include <iostream>
#include <map>
#include <string>
#include <vector>

// every header the reference's headers pull in, first, so that the access
// override below reaches the reference's two classes only
#include "Partio.h"
#include "cuda_runtime.h"
#include "cufft.h"
#include "device_launch_parameters.h"
#include "helper_cuda.h"
#include "helper_functions.h"
#include "opencv2/opencv.hpp"
#include "vectorUtil.cuh"

#define private public
#include "KaminoSolver.cuh"
#undef private

KaminoQuantity::KaminoQuantity(std::string attributeName, size_t nPhi, size_t nTheta, fReal phiOffset,
                               fReal thetaOffset)
    : attrName(attributeName), nPhi(nPhi), nTheta(nTheta), gridLen(M_2PI / nPhi), invGridLen(1.0 / gridLen),
      phiOffset(phiOffset), thetaOffset(thetaOffset), cpuBuffer(new fReal[nPhi * nTheta]), gpuThisStep(nullptr),
      thisStepPitch(0), gpuNextStep(nullptr), nextStepPitch(0)
{
    std::memset(cpuBuffer, 0, sizeof(fReal) * nPhi * nTheta);
}

KaminoQuantity::~KaminoQuantity() { delete[] cpuBuffer; }
size_t KaminoQuantity::getNPhi() { return nPhi; }
size_t KaminoQuantity::getNTheta() { return nTheta; }
fReal& KaminoQuantity::accessCPUValueAt(size_t phi, size_t theta) { return cpuBuffer[theta * nPhi + phi]; }
void KaminoQuantity::setCPUValueAt(size_t phi, size_t theta, fReal val) { accessCPUValueAt(phi, theta) = val; }

KaminoSolver::KaminoSolver(size_t nPhi, size_t nTheta, fReal radius, fReal frameDuration, fReal A, int B, int C,
                           int D, int E)
    : nPhi(nPhi), nTheta(nTheta), radius(radius), gridLen(M_2PI / nPhi), invGridLen(1.0 / gridLen),
      A(A), B(B), C(C), D(D), E(E), frameDuration(frameDuration), timeStep(0.0), timeElapsed(0.0)
{
    velPhi = new KaminoQuantity("velPhi", nPhi, nTheta, vPhiPhiOffset, vPhiThetaOffset);
    velTheta = new KaminoQuantity("velTheta", nPhi, nTheta - 1, vThetaPhiOffset, vThetaThetaOffset);
    pressure = density = nullptr;
    particles = nullptr;
}

KaminoSolver::~KaminoSolver()
{
    delete velPhi;
    delete velTheta;
}

void KaminoSolver::copyVelocity2GPU() {}

// u_phi [nt][2 nt] and u_theta [nt-1][2 nt] as initialize_velocity leaves
// them for a sphere of n_theta rows and the given radius.
extern "C" int ref_fbm_velocity(int n_theta, float radius, float* u_phi, float* u_theta)
{
    if (n_theta < 2 || !u_phi || !u_theta) return -1;
    const size_t nt = (size_t)n_theta, np = 2 * nt;
    KaminoSolver s(np, nt, radius, 0.005f, 0.0f, 1, 1, 1, 1);
    s.initialize_velocity();
    std::memcpy(u_phi, s.velPhi->cpuBuffer, sizeof(float) * np * nt);
    std::memcpy(u_theta, s.velTheta->cpuBuffer, sizeof(float) * np * (nt - 1));
    return 0;
}
