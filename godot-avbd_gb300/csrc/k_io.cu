// Body state exchange with the host: the Rigid public fields positionLin, positionAng,
// velocityLin, velocityAng (src/avbd/types.hpp:79-88) travel as one contiguous SoA block
// [pos 3n | quat 4n | vel 3n | angvel 3n] so an upload or download is a single copy.

#include "kernels.cuh"
#include "prims.cuh"

namespace avbdg {

namespace {

__global__ void packStateKernel(Dev d, int first, int count, float *out) {
    pdlWait();
    pdlTrigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count)
        return;
    const int g = first + i;
    const real4 x = d.x[g], q = d.q[g], v = d.v[g], w = d.w[g];
    float *p = out, *o = out + 3 * count, *vv = out + 7 * count, *ww = out + 10 * count;
    p[3 * i] = x.x;
    p[3 * i + 1] = x.y;
    p[3 * i + 2] = x.z;
    o[4 * i] = q.x;
    o[4 * i + 1] = q.y;
    o[4 * i + 2] = q.z;
    o[4 * i + 3] = q.w;
    vv[3 * i] = v.x;
    vv[3 * i + 1] = v.y;
    vv[3 * i + 2] = v.z;
    ww[3 * i] = w.x;
    ww[3 * i + 1] = w.y;
    ww[3 * i + 2] = w.z;
}

// Sets *bad when an uploaded position or velocity component is not finite (orientations are taken
// as given, as the host-side check does).
__global__ void checkStateKernel(int count, const float *in, int mask, int *bad) {
    pdlWait();
    pdlTrigger();
    const long long total = 13LL * count;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < total; k += stride) {
        const int field = k < 3LL * count ? 1 : (k < 7LL * count ? 2 : (k < 10LL * count ? 4 : 8));
        if ((mask & field) && field != 2 && !isfinite(in[k]))
            *bad = 1;
    }
}

// Fields not in `mask` (1 pos, 2 quat, 4 vel, 8 angvel) keep their device values; the packed
// companions (mass in x.w, gravity in v.w) are preserved. With `bad` set nothing is written.
__global__ void unpackStateKernel(Dev d, int first, int count, const float *in, int mask, const int *bad) {
    pdlWait();
    pdlTrigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count || (bad && *bad))
        return;
    const int g = first + i;
    const float *p = in, *o = in + 3 * count, *vv = in + 7 * count, *ww = in + 10 * count;
    if (mask & 1) {
        const real4 x = d.x[g];
        d.x[g] = mk4(p[3 * i], p[3 * i + 1], p[3 * i + 2], x.w);
    }
    if (mask & 2)
        d.q[g] = mk4(o[4 * i], o[4 * i + 1], o[4 * i + 2], o[4 * i + 3]);
    if (mask & 4) {
        const real4 v = d.v[g];
        d.v[g] = mk4(vv[3 * i], vv[3 * i + 1], vv[3 * i + 2], v.w);
    }
    if (mask & 8)
        d.w[g] = mk4(ww[3 * i], ww[3 * i + 1], ww[3 * i + 2], 0.0f);
}

} // namespace

void launchPackState(const Dev &d, int first, int count, float *out, cudaStream_t s) {
    ++launchCount();
    launchK(packStateKernel, divUp(count > 0 ? count : 1, 256), 256, 0, s, d, first, count, out);
}

void launchCheckState(int count, const float *in, int mask, int *bad, cudaStream_t s) {
    ++launchCount();
    launchK(checkStateKernel, residentGrid(checkStateKernel, 256, divUp(13 * (count > 0 ? count : 1), 256)), 256, 0, s, 
            count, in, mask, bad);
}

void launchUnpackState(const Dev &d, int first, int count, const float *in, int mask, const int *bad,
                       cudaStream_t s) {
    ++launchCount();
    launchK(unpackStateKernel, divUp(count > 0 ? count : 1, 256), 256, 0, s, d, first, count, in, mask, bad);
}

} // namespace avbdg
