// knn.cuh - the warp's running k-nearest list (k <= 64), shared by the tree
// walk, the exhaustive sweeps and the roadmap planner.  Entry j lives in lane
// j (ld0/li0, j < 32) or lane j - 32 (ld1/li1), sorted by (distance, id);
// tau is the k-th distance once the list is full, else the radius.
#pragma once
#include "common.cuh"

// the lanes with cand set offer (dd, pid) to the list, lowest lane first
__device__ __forceinline__ void knn_insert(int lane, int k, double radius, bool cand, double dd, int pid, double& ld0,
                                           double& ld1, int& li0, int& li1, int& cnt, double& tau, float& tauf) {
    unsigned cmask = __ballot_sync(0xffffffffu, cand);
    while (cmask) {
        int src = __ffs(cmask) - 1;
        cmask &= cmask - 1;
        double cd = __shfl_sync(0xffffffffu, dd, src);
        int ci = __shfl_sync(0xffffffffu, pid, src);
        // insert (cd, ci) into the sorted list if it ranks among the k best
        if (cnt == k) {
            double kd = (k - 1) < 32 ? __shfl_sync(0xffffffffu, ld0, k - 1) : __shfl_sync(0xffffffffu, ld1, k - 33);
            int ki = (k - 1) < 32 ? __shfl_sync(0xffffffffu, li0, k - 1) : __shfl_sync(0xffffffffu, li1, k - 33);
            if (!(cd < kd || (cd == kd && ci < ki))) continue;
        }
        // rank position = number of entries strictly ahead of (cd, ci)
        bool ahead0 = lane < cnt && (ld0 < cd || (ld0 == cd && li0 < ci));
        bool ahead1 = lane + 32 < cnt && (ld1 < cd || (ld1 == cd && li1 < ci));
        int pos = __popc(__ballot_sync(0xffffffffu, ahead0)) + __popc(__ballot_sync(0xffffffffu, ahead1));
        // shift entries at >= pos one place back
        double p0d = __shfl_up_sync(0xffffffffu, ld0, 1);
        int p0i = __shfl_up_sync(0xffffffffu, li0, 1);
        double p1d = __shfl_up_sync(0xffffffffu, ld1, 1);
        int p1i = __shfl_up_sync(0xffffffffu, li1, 1);
        double last0d = __shfl_sync(0xffffffffu, ld0, 31);
        int last0i = __shfl_sync(0xffffffffu, li0, 31);
        if (lane == 0) { p1d = last0d; p1i = last0i; }
        // slot 0 entries (index = lane)
        if (lane > pos) { ld0 = p0d; li0 = p0i; }
        else if (lane == pos) { ld0 = cd; li0 = ci; }
        int j1 = lane + 32;
        if (j1 > pos) { ld1 = p1d; li1 = p1i; }
        else if (j1 == pos) { ld1 = cd; li1 = ci; }
        if (cnt < k) ++cnt;
        if (cnt == k) {
            double kd = (k - 1) < 32 ? __shfl_sync(0xffffffffu, ld0, k - 1) : __shfl_sync(0xffffffffu, ld1, k - 33);
            tau = fmin(kd, radius);
            tauf = __double2float_ru(tau);
        }
    }
}
