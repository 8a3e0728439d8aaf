// pk_engine_host.cuh — device buffers and the launch sequence of one world step.
//
// Included by pk_engine_f64.cu (FP64, -fmad=false: the parity form) and pk_engine_f32.cu (FP32 bulk
// arithmetic with FP64 accumulated impulses: the precision form).
#pragma once

#include "pk_engine.cuh"
#include "pk_engine_api.h"

#include <cstring>
#include <cuda_runtime.h>
#include <deque>

namespace pk
{

// Page-locked host staging mirrored by device memory, for uploads that must not wait for the GPU
// (the serving loop admits and retires worlds while earlier steps run). Regions are handed out in
// ring order; a region is reused only after the event recorded behind its last use has completed.
class StagingRing
{
public:
    cudaError_t init(size_t bytes)
    {
        cudaError_t e = cudaHostAlloc(reinterpret_cast<void **>(&host_), bytes, cudaHostAllocDefault);
        if (e != cudaSuccess) return e;
        e = cudaMalloc(reinterpret_cast<void **>(&dev_), bytes);
        if (e != cudaSuccess) return e;
        cap_ = bytes;
        return cudaSuccess;
    }
    void release()
    {
        for (Region &r : busy_) cudaEventDestroy(r.ev);
        for (cudaEvent_t e : spare_) cudaEventDestroy(e);
        busy_.clear();
        spare_.clear();
        if (host_) cudaFreeHost(host_);
        if (dev_) cudaFree(dev_);
        host_ = dev_ = nullptr;
        cap_ = head_ = 0;
    }
    bool ready() const { return cap_ > 0; }
    // n bytes at a 256-byte aligned offset; waits only for earlier users of the same bytes
    cudaError_t reserve(size_t n, size_t *off)
    {
        n = (n + 255) & ~size_t(255);
        if (n > cap_) return cudaErrorMemoryAllocation;
        size_t s = head_;
        if (s + n > cap_) s = 0;
        for (auto it = busy_.begin(); it != busy_.end();)
        {
            const bool overlap = it->lo < s + n && s < it->hi;
            if (overlap || cudaEventQuery(it->ev) == cudaSuccess)
            {
                cudaError_t e = cudaEventSynchronize(it->ev);
                if (e != cudaSuccess) return e;
                spare_.push_back(it->ev);
                it = busy_.erase(it);
            }
            else
                ++it;
        }
        *off = s;
        head_ = s + n;
        pending_lo_ = s;
        pending_hi_ = s + n;
        return cudaSuccess;
    }
    // the last reserved region is in use by the work enqueued on `st` up to now
    cudaError_t commit(cudaStream_t st)
    {
        cudaEvent_t ev;
        if (!spare_.empty())
        {
            ev = spare_.back();
            spare_.pop_back();
        }
        else
        {
            cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            if (e != cudaSuccess) return e;
        }
        cudaError_t e = cudaEventRecord(ev, st);
        if (e != cudaSuccess) return e;
        busy_.push_back(Region{pending_lo_, pending_hi_, ev});
        return cudaSuccess;
    }
    unsigned char *host(size_t off) const { return host_ + off; }
    unsigned char *dev(size_t off) const { return dev_ + off; }

private:
    struct Region
    {
        size_t lo, hi;
        cudaEvent_t ev;
    };
    unsigned char *host_ = nullptr, *dev_ = nullptr;
    size_t cap_ = 0, head_ = 0, pending_lo_ = 0, pending_hi_ = 0;
    std::deque<Region> busy_;
    std::vector<cudaEvent_t> spare_;
};

// Sub-array offsets inside one staging region (each 256-byte aligned).
struct StageLayout
{
    size_t total = 0;
    size_t add(size_t bytes)
    {
        size_t o = total;
        total += (bytes + 255) & ~size_t(255);
        return o;
    }
};

#define PK_CUDA(x)                                                                                     \
    do                                                                                                 \
    {                                                                                                  \
        cudaError_t e_ = (x);                                                                          \
        if (e_ != cudaSuccess)                                                                         \
        {                                                                                              \
            last_err_ = int(e_);                                                                       \
            std::fprintf(stderr, "physkit_gb300: %s failed: %s\n", #x, cudaGetErrorString(e_));        \
            return -int(e_) - 1000;                                                                    \
        }                                                                                              \
    } while (0)

template <class T> __device__ __forceinline__ void refresh_one(Dev<T> d, int s)
{
    // particle::update_derived_state (particle.h:140-146)
    Qt<T> q = ldq(d.pose[s].q);
    M3<T> R = to_matrix(q), Rt = transpose(R);
    M3<T> il, ili;
    for (int k = 0; k < 9; ++k)
    {
        il.m[k] = d.prm[s].il[k];
        ili.m[k] = d.prm[s].il_inv[k];
    }
    M3<T> iw = matmul(matmul(R, il), Rt);
    M3<T> iwi = matmul(matmul(R, ili), Rt);
    for (int k = 0; k < 9; ++k)
    {
        d.iw[9 * s + k] = iw.m[k];
        d.iwinv[9 * s + k] = iwi.m[k];
    }
}

template <class T>
__global__ void k_install_bodies(Dev<T> d, const int *slots, const Pose<T> *pose, const Vel<T> *vel,
                                 const Params<T> *prm, const Meta *meta, int n)
{
    PK_GRID_STRIDE(i, n)
    {
        int s = slots[i];
        d.pose[s] = pose[i];
        d.vel[s] = vel[i];
        d.prm[s] = prm[i];
        d.meta[s] = meta[i];
        // dynamic_bvh::add stores the exact (not fattened) bounds (bvh.h:294-302)
        d.tbox[s] = world_bounds(d.shape_box[meta[i].shape], ldq(pose[i].q), ld3(pose[i].p));
        refresh_one(d, s);
    }
}

template <class T> __global__ void k_refresh_derived(Dev<T> d, int first, int n)
{
    PK_GRID_STRIDE(i, n) refresh_one(d, first + i);
}

template <class T> __global__ void k_kill_body(Dev<T> d, int slot) { d.meta[slot].flags = 0; }

// Read-back rows (particle.h:135-149): pos3 quat4 vel3 ang_vel3 alive, 14 doubles per slot; an
// empty slot reads as zeros.
template <class T> __global__ void k_pack_bodies(Dev<T> d, double *__restrict__ out, int n)
{
    PK_GRID_STRIDE(i, n)
    {
        double *o = out + 14 * size_t(i);
        if (!(d.meta[i].flags & BODY_ALIVE))
        {
            for (int k = 0; k < 14; ++k) o[k] = 0.0;
            continue;
        }
        const Pose<T> ps = d.pose[i];
        const Vel<T> ve = d.vel[i];
        for (int k = 0; k < 3; ++k)
        {
            o[k] = double(ps.p[k]);
            o[7 + k] = double(ve.v[k]);
            o[10 + k] = double(ve.w[k]);
        }
        for (int k = 0; k < 4; ++k) o[3 + k] = double(ps.q[k]);
        o[13] = 1.0;
    }
}

static __global__ void k_zero_ints(int *p, int n)
{
    PK_GRID_STRIDE(i, n) p[i] = 0;
}

template <class T> class Engine final : public EngineBase
{
public:
    ~Engine() override { release(); }

    int precision_bits() const override { return int(sizeof(T) * 8); }
    int last_error() const override { return last_err_; }
    void *stream() override { return st_; }

    int init(const EngineConfig &cfg) override
    {
        cfg_ = cfg;
        int dev = 0;
        PK_CUDA(cudaGetDevice(&dev));
        PK_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
        PK_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
        PK_CUDA(cudaStreamCreateWithFlags(&st2_, cudaStreamNonBlocking));
        PK_CUDA(cudaStreamCreateWithFlags(&st3_, cudaStreamNonBlocking));
        PK_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
        PK_CUDA(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming));
        PK_CUDA(cudaEventCreateWithFlags(&join3_, cudaEventDisableTiming));
        PK_CUDA(cudaStreamCreateWithFlags(&cs_, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k)
        {
            PK_CUDA(cudaEventCreateWithFlags(&packed_[k], cudaEventDisableTiming));
            PK_CUDA(cudaEventCreateWithFlags(&copied_[k], cudaEventDisableTiming));
        }
        const size_t N = size_t(cfg.body_cap), P = size_t(cfg.pair_cap), W = size_t(cfg.max_worlds);
        const size_t CC = size_t(cfg.contact_cap > 0 && cfg.contact_cap < cfg.pair_cap ? cfg.contact_cap : cfg.pair_cap);
        Dev<T> &d = d_;
        std::memset(&d, 0, sizeof(d));
        d.max_worlds = cfg.max_worlds;
        d.pair_cap = cfg.pair_cap;
        d.contact_cap = int(CC);
        d.lbits = cfg.lbits;
        d.wbits = cfg.wbits;
        d.iterations = cfg.iterations;
        PK_CUDA(alloc(&d.pose, N));
        PK_CUDA(alloc(&d.vel, N));
        PK_CUDA(alloc(&d.iw, 9 * N));
        PK_CUDA(alloc(&d.iwinv, 9 * N));
        PK_CUDA(alloc(&d.prm, N));
        PK_CUDA(alloc(&d.tbox, N));
        PK_CUDA(alloc(&d.meta, N));
        PK_CUDA(cudaMemset(d.meta, 0, sizeof(Meta) * N));
        PK_CUDA(alloc(&counters_, 32));
        PK_CUDA(cudaMemset(counters_, 0, sizeof(int) * 32));
        d.nslots = counters_ + 0;
        d.nleaf = counters_ + 1;
        d.npairs = counters_ + 2;
        d.npairs_old = counters_ + 3;
        d.status = counters_ + 4;
        d.epoch = counters_ + 5;
        d.gjk_count = counters_ + 6;
        d.epa_count = counters_ + 7;
        d.gjk_count_heavy = counters_ + 8;
        d.epa_count_heavy = counters_ + 9;
        d.np_iters = reinterpret_cast<unsigned long long *>(counters_ + 10); // counters 10..15
        d.np_verts = reinterpret_cast<unsigned long long *>(counters_ + 24); // counters 24..25
        d.nnew = counters_ + 16;
        d.njoints = counters_ + 17; // zero until joints are set
        d.ccount = counters_ + 18;
        d.gjk2_count = counters_ + 19;
        d.gjk2_count_heavy = counters_ + 20;
        d.all_small = counters_ + 21;
        d.epa_total = counters_ + 22;
        PK_CUDA(alloc(&d.jstart, W));
        PK_CUDA(alloc(&d.jend, W));
        PK_CUDA(cudaMemset(d.jstart, 0, sizeof(int) * W));
        PK_CUDA(cudaMemset(d.jend, 0, sizeof(int) * W));
        int minus1 = -1;
        PK_CUDA(cudaMemcpy(d.epoch, &minus1, sizeof(int), cudaMemcpyHostToDevice));
        PK_CUDA(alloc(&d.wp, W));
        PK_CUDA(cudaMemset(d.wp, 0, sizeof(WorldParams<T>) * W));
        PK_CUDA(alloc(&d.wbounds, 6 * W));
        PK_CUDA(alloc(&d.wroot, W));
        PK_CUDA(alloc(&d.wleaf_lo, W));
        PK_CUDA(alloc(&d.wleaf_hi, W));
        PK_CUDA(alloc(&d.wlive, W));
        PK_CUDA(alloc(&d.mstart, W));
        PK_CUDA(alloc(&d.mend, W));
        PK_CUDA(alloc(&d.mstart_old, W));
        PK_CUDA(alloc(&d.mend_old, W));
        PK_CUDA(alloc(&d.nstart, W));
        PK_CUDA(alloc(&d.nend, W));
        PK_CUDA(cudaMemset(d.mstart_old, 0, sizeof(int) * W));
        PK_CUDA(cudaMemset(d.mend_old, 0, sizeof(int) * W));
        PK_CUDA(alloc(&d.ncolours, W));
        PK_CUDA(cudaMemset(d.ncolours, 0, sizeof(int) * W));
        {
            int *wo, *wn;
            PK_CUDA(alloc(&wo, W));
            PK_CUDA(alloc(&wn, W));
            std::vector<int> ident(W);
            for (size_t i = 0; i < W; ++i) ident[i] = int(i);
            PK_CUDA(cudaMemcpy(wo, ident.data(), sizeof(int) * W, cudaMemcpyHostToDevice));
            PK_CUDA(cudaMemset(wn, 0x7F, sizeof(int) * W)); // "too large to cache" until set
            d.world_order = wo;
            d.world_nlocal = wn;
            PK_CUDA(alloc(&goff_dev_, W + 1));
        }
        PK_CUDA(radix_sort_prepare<uint64_t>());
        PK_CUDA(cudaFuncSetAttribute(k_broad_small<T, kBroadClasses[0].minn, kBroadClasses[0].maxn,
                                                   kBroadClasses[0].qcap, kBroadClasses[0].threads>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(broad_smem_bytes<kBroadClasses[0].maxn, kBroadClasses[0].qcap>())));
        PK_CUDA(cudaFuncSetAttribute(k_broad_small<T, kBroadClasses[1].minn, kBroadClasses[1].maxn,
                                                   kBroadClasses[1].qcap, kBroadClasses[1].threads>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(broad_smem_bytes<kBroadClasses[1].maxn, kBroadClasses[1].qcap>())));
        PK_CUDA(cudaFuncSetAttribute(k_broad_small<T, kBroadClasses[2].minn, kBroadClasses[2].maxn,
                                                   kBroadClasses[2].qcap, kBroadClasses[2].threads>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(broad_smem_bytes<kBroadClasses[2].maxn, kBroadClasses[2].qcap>())));
        PK_CUDA(cudaFuncSetAttribute(k_solve_world<T, 256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(kMaxSolveSmem)));
        PK_CUDA(cudaFuncSetAttribute(k_solve_group<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMaxSolveSmem)));
        PK_CUDA(cudaFuncSetAttribute(k_solve_group<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMaxSolveSmem)));
        PK_CUDA(cudaFuncSetAttribute(k_solve_world<T, 256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(kMaxSolveSmem)));
        PK_CUDA(cudaFuncSetAttribute(k_solve_world<T, solve_max_threads<T>(), false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMaxSolveSmem)));
        PK_CUDA(cudaFuncSetAttribute(k_solve_world<T, solve_max_threads<T>(), true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMaxSolveSmem)));
        {
            int per_sm = 0;
            PK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_grid<T>, 256, 0));
            grid_blocks_ = sms_ * (per_sm > 0 ? per_sm : 1);
            PK_CUDA(cudaMalloc(&grid_scratch_, sizeof(GridScratch)));
        }
        for (int k = 0; k < 2; ++k)
        {
            PK_CUDA(alloc(&mkey_[k], N));
            PK_CUDA(alloc(&mval_[k], N));
            PK_CUDA(alloc(&pkey_[k], P));
            PK_CUDA(alloc(&pval_[k], P));
            PK_CUDA(alloc(&man_[k], P));
        }
        PK_CUDA(alloc(&d.nodes, 4 * N));
        PK_CUDA(alloc(&d.parent, N));
        PK_CUDA(alloc(&d.leaf_parent, N));
        PK_CUDA(alloc(&d.refit_flag, N));
        PK_CUDA(alloc(&d.key_old, P));
        PK_CUDA(alloc(&d.val_old, P));
        PK_CUDA(alloc(&d.event, P));
        PK_CUDA(alloc(&d.old_idx, P));
        PK_CUDA(alloc(&d.gjk_list, P));
        PK_CUDA(alloc(&d.clist, P));
        PK_CUDA(alloc(&d.gjk_list2, P));
        PK_CUDA(alloc(&d.gcls, 3 * kPairClasses));
        PK_CUDA(cudaMemset(d.gcls, 0, sizeof(int) * 3 * kPairClasses));
        PK_CUDA(alloc(&d.epa_list, CC));
        PK_CUDA(alloc(&d.epa_simplex, CC));
        PK_CUDA(alloc(&d.rowidx, P));
        PK_CUDA(alloc(&d.rows, 4 * CC));
        PK_CUDA(alloc(&d.racc, 12 * CC));
        if (sizeof(T) == 4) PK_CUDA(alloc(&d.raccf, 12 * CC));
        if (sizeof(T) == 4) PK_CUDA(alloc(&d.rdel, 12 * CC));
        PK_CUDA(alloc(&d.rowmask, P));
        PK_CUDA(alloc(&d.colour, P));
        PK_CUDA(alloc(&d.colour_tmp, P));
        PK_CUDA(alloc(&d.pair_colour, P));
        PK_CUDA(alloc(&d.order, P));
        PK_CUDA(alloc(&d.srec, P));
        PK_CUDA(alloc(&d.crec, P));
        PK_CUDA(alloc(&d.owner, N));
        PK_CUDA(alloc(&d.used, N));
        int hb = cfg.sort_blocks_bodies > cfg.sort_blocks_pairs ? cfg.sort_blocks_bodies : cfg.sort_blocks_pairs;
        PK_CUDA(alloc(&hist_, size_t(kSortRadix) * (hb + 1))); // digit table + one row of digit totals
        PK_CUDA(alloc(&d.verts, 3 * size_t(cfg.vert_cap > 0 ? cfg.vert_cap : 1)));
        if (sizeof(T) == 8)
        {
            PK_CUDA(alloc(&d.verts32, 3 * size_t(cfg.vert_cap > 0 ? cfg.vert_cap : 1)));
            PK_CUDA(alloc(&d.shape32, 8 * size_t(cfg.shape_cap > 0 ? cfg.shape_cap : 1)));
            PK_CUDA(alloc(&d.pose32, 2 * size_t(N)));
        }
        PK_CUDA(alloc(&shape_range_, size_t(cfg.shape_cap > 0 ? cfg.shape_cap : 1)));
        PK_CUDA(alloc(&shape_box_, size_t(cfg.shape_cap > 0 ? cfg.shape_cap : 1)));
        PK_CUDA(alloc(&shape_rmax_, size_t(cfg.shape_cap > 0 ? cfg.shape_cap : 1)));
        d.shape_range = shape_range_;
        d.shape_box = shape_box_;
        d.shape_rmax = shape_rmax_;
        d.man_old = man_[0];
        d.man_new = man_[1];
        PK_CUDA(cudaDeviceSynchronize());
        return 0;
    }

    int set_shapes(const std::vector<double> &verts, const std::vector<int> &ranges,
                   const std::vector<double> &boxes, const std::vector<double> &clusters,
                   const std::vector<double> &rmax) override
    {
        size_t nv = verts.size() / 3, ns = ranges.size() / 8, nc = clusters.size() / 4;
        if (nv > size_t(cfg_.vert_cap) || ns > size_t(cfg_.shape_cap)) return -3;
        std::vector<T> v(verts.size());
        for (size_t i = 0; i < verts.size(); ++i) v[i] = T(verts[i]);
        std::vector<Aabb<T>> b(ns);
        for (size_t i = 0; i < ns; ++i)
            b[i] = Aabb<T>{{T(boxes[6 * i]), T(boxes[6 * i + 1]), T(boxes[6 * i + 2])},
                           {T(boxes[6 * i + 3]), T(boxes[6 * i + 4]), T(boxes[6 * i + 5])}};
        std::vector<T> c(clusters.size() > 0 ? clusters.size() : 4);
        for (size_t i = 0; i < clusters.size(); ++i) c[i] = T(clusters[i]);
        std::vector<T> r(ns);
        for (size_t i = 0; i < ns; ++i) r[i] = T(rmax[i]);
        if (nc > clusters_cap_)
        {
            if (clusters_) cudaFree(clusters_);
            clusters_cap_ = nc + nc / 2 + 16;
            PK_CUDA(cudaMalloc(&clusters_, sizeof(T) * 4 * clusters_cap_));
        }
        d_.clusters = clusters_;
        PK_CUDA(cudaMemcpyAsync(const_cast<T *>(d_.verts), v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st_));
        std::vector<float> v32(verts.size());
        std::vector<float> s32(8 * ns);
        if (d_.verts32)
        {
            for (size_t i = 0; i < verts.size(); ++i) v32[i] = float(verts[i]);
            PK_CUDA(cudaMemcpyAsync(const_cast<float *>(d_.verts32), v32.data(), sizeof(float) * v32.size(),
                                    cudaMemcpyHostToDevice, st_));
            for (size_t i = 0; i < ns; ++i)
            {
                for (int k = 0; k < 6; ++k) s32[8 * i + k] = float(boxes[6 * i + k]);
                s32[8 * i + 6] = float(T(rmax[i]));
                s32[8 * i + 7] = 0.0f;
            }
            if (ns) PK_CUDA(cudaMemcpyAsync(const_cast<float *>(d_.shape32), s32.data(), sizeof(float) * s32.size(),
                                            cudaMemcpyHostToDevice, st_));
        }
        PK_CUDA(cudaMemcpyAsync(shape_range_, ranges.data(), sizeof(int) * ranges.size(), cudaMemcpyHostToDevice, st_));
        PK_CUDA(cudaMemcpyAsync(shape_box_, b.data(), sizeof(Aabb<T>) * ns, cudaMemcpyHostToDevice, st_));
        PK_CUDA(cudaMemcpyAsync(shape_rmax_, r.data(), sizeof(T) * ns, cudaMemcpyHostToDevice, st_));
        if (nc) PK_CUDA(cudaMemcpyAsync(clusters_, c.data(), sizeof(T) * 4 * nc, cudaMemcpyHostToDevice, st_));
        PK_CUDA(cudaStreamSynchronize(st_));
        return 0;
    }

    int set_world(int w, const double g[3], double gnorm, int active) override
    {
        WorldParams<T> p;
        p.g[0] = T(g[0]);
        p.g[1] = T(g[1]);
        p.g[2] = T(g[2]);
        p.gnorm = T(gnorm);
        p.active = active;
        p.pad = 0;
        PK_CUDA(cudaMemcpyAsync(d_.wp + w, &p, sizeof(p), cudaMemcpyHostToDevice, st_));
        PK_CUDA(cudaStreamSynchronize(st_));
        return 0;
    }

    // The same upload without waiting for the GPU: staged through pinned memory and enqueued on
    // the world's stream behind the steps already in flight.
    int upload_bodies_async(const int *slots, const HostBody *b, int n, int nslots) override
    {
        PK_CUDA(ensure_staging());
        StageLayout L;
        const size_t o_sl = L.add(sizeof(int) * size_t(n)), o_pose = L.add(sizeof(Pose<T>) * size_t(n)),
                     o_vel = L.add(sizeof(Vel<T>) * size_t(n)), o_prm = L.add(sizeof(Params<T>) * size_t(n)),
                     o_meta = L.add(sizeof(Meta) * size_t(n)), o_ns = L.add(sizeof(int));
        size_t base = 0;
        PK_CUDA(stage_.reserve(L.total, &base));
        unsigned char *h = stage_.host(base), *dv = stage_.dev(base);
        int *sl = reinterpret_cast<int *>(h + o_sl);
        Pose<T> *pose = reinterpret_cast<Pose<T> *>(h + o_pose);
        Vel<T> *vel = reinterpret_cast<Vel<T> *>(h + o_vel);
        Params<T> *prm = reinterpret_cast<Params<T> *>(h + o_prm);
        Meta *meta = reinterpret_cast<Meta *>(h + o_meta);
        for (int i = 0; i < n; ++i)
        {
            sl[i] = slots[i];
            convert_body(b[i], pose[i], vel[i], prm[i], meta[i]);
        }
        *reinterpret_cast<int *>(h + o_ns) = nslots;
        PK_CUDA(cudaMemcpyAsync(dv, h, L.total, cudaMemcpyHostToDevice, st_));
        if (n > 0)
            k_install_bodies<T><<<grid(n), 256, 0, st_>>>(d_, reinterpret_cast<const int *>(dv + o_sl),
                                                          reinterpret_cast<const Pose<T> *>(dv + o_pose),
                                                          reinterpret_cast<const Vel<T> *>(dv + o_vel),
                                                          reinterpret_cast<const Params<T> *>(dv + o_prm),
                                                          reinterpret_cast<const Meta *>(dv + o_meta), n);
        PK_CUDA(cudaGetLastError());
        PK_CUDA(cudaMemcpyAsync(const_cast<int *>(d_.nslots), dv + o_ns, sizeof(int), cudaMemcpyDeviceToDevice, st_));
        PK_CUDA(stage_.commit(st_));
        nslots_ = nslots;
        return 0;
    }

    static void convert_body(const HostBody &h, Pose<T> &pose, Vel<T> &vel, Params<T> &prm, Meta &meta)
    {
        for (int k = 0; k < 3; ++k)
        {
            pose.p[k] = T(h.pos[k]);
            vel.v[k] = T(h.vel[k]);
            vel.w[k] = T(h.ang_vel[k]);
        }
        for (int k = 0; k < 4; ++k) pose.q[k] = T(h.quat[k]);
        prm.mass = T(h.mass);
        prm.inv_mass = T(h.inv_mass);
        prm.restitution = T(h.restitution);
        prm.friction = T(h.friction);
        for (int k = 0; k < 9; ++k)
        {
            prm.il[k] = T(h.il[k]);
            prm.il_inv[k] = T(h.il_inv[k]);
        }
        meta = Meta{uint32_t(h.world), uint32_t(h.local), uint32_t(h.shape), uint32_t(h.flags), h.created, -1};
    }

    int upload_bodies(const int *slots, const HostBody *b, int n, int nslots) override
    {
        if (n > 0)
        {
            std::vector<int> sl(slots, slots + n);
            std::vector<Pose<T>> pose(n);
            std::vector<Vel<T>> vel(n);
            std::vector<Params<T>> prm(n);
            std::vector<Meta> meta(n);
            for (int i = 0; i < n; ++i) convert_body(b[i], pose[i], vel[i], prm[i], meta[i]);
            int *dsl;
            Pose<T> *dpose;
            Vel<T> *dvel;
            Params<T> *dprm;
            Meta *dmeta;
            PK_CUDA(cudaMallocAsync(&dsl, sizeof(int) * n, st_));
            PK_CUDA(cudaMallocAsync(&dpose, sizeof(Pose<T>) * n, st_));
            PK_CUDA(cudaMallocAsync(&dvel, sizeof(Vel<T>) * n, st_));
            PK_CUDA(cudaMallocAsync(&dprm, sizeof(Params<T>) * n, st_));
            PK_CUDA(cudaMallocAsync(&dmeta, sizeof(Meta) * n, st_));
            PK_CUDA(cudaMemcpyAsync(dsl, sl.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st_));
            PK_CUDA(cudaMemcpyAsync(dpose, pose.data(), sizeof(Pose<T>) * n, cudaMemcpyHostToDevice, st_));
            PK_CUDA(cudaMemcpyAsync(dvel, vel.data(), sizeof(Vel<T>) * n, cudaMemcpyHostToDevice, st_));
            PK_CUDA(cudaMemcpyAsync(dprm, prm.data(), sizeof(Params<T>) * n, cudaMemcpyHostToDevice, st_));
            PK_CUDA(cudaMemcpyAsync(dmeta, meta.data(), sizeof(Meta) * n, cudaMemcpyHostToDevice, st_));
            k_install_bodies<T><<<grid(n), 256, 0, st_>>>(d_, dsl, dpose, dvel, dprm, dmeta, n);
            PK_CUDA(cudaGetLastError());
            PK_CUDA(cudaFreeAsync(dsl, st_));
            PK_CUDA(cudaFreeAsync(dpose, st_));
            PK_CUDA(cudaFreeAsync(dvel, st_));
            PK_CUDA(cudaFreeAsync(dprm, st_));
            PK_CUDA(cudaFreeAsync(dmeta, st_));
        }
        nslots_ = nslots;
        PK_CUDA(cudaMemcpyAsync(const_cast<int *>(d_.nslots), &nslots_, sizeof(int), cudaMemcpyHostToDevice, st_));
        PK_CUDA(cudaStreamSynchronize(st_));
        return 0;
    }

    int set_world_order_async(const int *order, const int *nlocal, int n) override
    {
        if (n != cfg_.max_worlds) return -3;
        PK_CUDA(ensure_staging());
        size_t base = 0;
        const size_t bytes = sizeof(int) * size_t(n);
        order_.assign(order, order + n);
        nlocal_.assign(nlocal, nlocal + n);
        split_worlds();
        const size_t gbytes = sizeof(int) * goff_.size();
        StageLayout L;
        const size_t o_ord = L.add(bytes), o_nl = L.add(bytes), o_g = L.add(gbytes);
        PK_CUDA(stage_.reserve(L.total, &base));
        std::memcpy(stage_.host(base + o_ord), order, bytes);
        std::memcpy(stage_.host(base + o_nl), nlocal, bytes);
        if (gbytes) std::memcpy(stage_.host(base + o_g), goff_.data(), gbytes);
        PK_CUDA(cudaMemcpyAsync(const_cast<int *>(d_.world_order), stage_.host(base + o_ord), bytes,
                                cudaMemcpyHostToDevice, st_));
        PK_CUDA(cudaMemcpyAsync(const_cast<int *>(d_.world_nlocal), stage_.host(base + o_nl), bytes,
                                cudaMemcpyHostToDevice, st_));
        if (gbytes) PK_CUDA(cudaMemcpyAsync(goff_dev_, stage_.host(base + o_g), gbytes, cudaMemcpyHostToDevice, st_));
        PK_CUDA(stage_.commit(st_));
        return 0;
    }

    int set_world_order(const int *order, const int *nlocal, int n) override
    {
        if (n != cfg_.max_worlds) return -3;
        PK_CUDA(cudaMemcpyAsync(const_cast<int *>(d_.world_order), order, sizeof(int) * n, cudaMemcpyHostToDevice, st_));
        PK_CUDA(cudaMemcpyAsync(const_cast<int *>(d_.world_nlocal), nlocal, sizeof(int) * n, cudaMemcpyHostToDevice, st_));
        order_.assign(order, order + n);
        nlocal_.assign(nlocal, nlocal + n);
        split_worlds();
        PK_CUDA(upload_groups());
        return 0;
    }

    // Worlds above tune_.small_world local indices get their own solver launch with a cache sized
    // for the largest world (if it fits in shared memory); the others share a small cache.
    void split_worlds()
    {
        big_worlds_ = 0;
        int maxl = 0;
        grid_worlds_.clear();
        for (size_t i = 0; i < order_.size(); ++i)
        {
            int nl = nlocal_[size_t(order_[i])];
            if (nl > kGridWorld)
            {
                grid_worlds_.push_back(order_[i]);
                continue;
            }
            if (nl > tune_.small_world) ++big_worlds_;
            maxl = nl > maxl ? nl : maxl;
        }
        // worlds handled by the grid solver sort first (largest first): skip them in the CTA launches
        big_worlds_ += int(grid_worlds_.size());
        int limit = int(kMaxSolveSmem / sizeof(Vel<T>));
        big_cache_ = maxl <= limit ? maxl : 0;
        // first-fit colouring keeps 16 bytes per local index in the same shared memory
        big_smem_ = sizeof(Vel<T>) * size_t(big_cache_);
        const size_t ff = 16 * size_t(maxl < kFirstFitMax ? maxl : kFirstFitMax);
        if (ff > big_smem_) big_smem_ = ff;
        // solve groups over the worlds after the large ones (in solve order, so sizes fall): up to
        // kGroupMax consecutive worlds while their local indices fit group_bodies; a larger world
        // is a group of its own. The groups are not used while the engine holds joints.
        goff_.clear();
        group_cache_ = 0;
        const int glimit = limit < tune_.group_bodies ? limit : tune_.group_bodies;
        if (glimit > 0 && !order_.empty())
        {
            const int n = int(order_.size());
            int i = big_worlds_;
            while (i < n)
            {
                goff_.push_back(i);
                int sum = 0, m = 0;
                const int mmax = tune_.group_warp ? (tune_.group_threads / 32 < kGroupMax ? tune_.group_threads / 32 : kGroupMax)
                                                  : kGroupMax;
                while (i < n && m < (mmax > 0 ? mmax : 1))
                {
                    const int nl = nlocal_[size_t(order_[size_t(i)])];
                    if (m > 0 && sum + nl > glimit) break;
                    sum += nl;
                    ++m;
                    ++i;
                }
                group_cache_ = sum > group_cache_ ? sum : group_cache_;
            }
            if (!goff_.empty()) goff_.push_back(n);
            if (group_cache_ > limit) goff_.clear(); // a single world above the cache (small_world > limit)
        }
    }
    int ngroups() const { return goff_.empty() ? 0 : int(goff_.size()) - 1; }
    cudaError_t upload_groups()
    {
        if (!goff_.empty())
        {
            cudaError_t e = cudaMemcpyAsync(goff_dev_, goff_.data(), sizeof(int) * goff_.size(), cudaMemcpyHostToDevice, st_);
            if (e != cudaSuccess) return e;
        }
        return cudaStreamSynchronize(st_);
    }

    int set_tunables(const Tunables &t) override
    {
        tune_ = t;
        // the small-world launch caches small_world bodies' velocities in shared memory
        const int limit = int(kMaxSolveSmem / sizeof(Vel<T>));
        if (tune_.small_world > limit) tune_.small_world = limit;
        split_worlds();
        PK_CUDA(upload_groups());
        return 0;
    }
    Tunables tunables() const override { return tune_; }

    int kill_world_async(const int *slots, int n, int world) override
    {
        Dev<T> d = d_;
        d.man_old = man_[parity_];
        if (n > 0)
        {
            PK_CUDA(ensure_staging());
            size_t base = 0;
            PK_CUDA(stage_.reserve(sizeof(int) * size_t(n), &base));
            std::memcpy(stage_.host(base), slots, sizeof(int) * size_t(n));
            PK_CUDA(cudaMemcpyAsync(stage_.dev(base), stage_.host(base), sizeof(int) * size_t(n),
                                    cudaMemcpyHostToDevice, st_));
            k_kill_bodies<T><<<grid(n), 256, 0, st_>>>(d, reinterpret_cast<const int *>(stage_.dev(base)), n);
            PK_CUDA(stage_.commit(st_));
        }
        k_purge_world<T><<<grid(cfg_.pair_cap), 256, 0, st_>>>(d, uint32_t(world));
        PK_CUDA(cudaGetLastError());
        return 0;
    }

    int set_active_mask_async(const uint8_t *mask, int n) override
    {
        if (n != cfg_.max_worlds) return -3;
        PK_CUDA(ensure_staging());
        size_t base = 0;
        PK_CUDA(stage_.reserve(size_t(n), &base));
        std::memcpy(stage_.host(base), mask, size_t(n));
        PK_CUDA(cudaMemcpyAsync(stage_.dev(base), stage_.host(base), size_t(n), cudaMemcpyHostToDevice, st_));
        k_set_active<T><<<grid(n), 256, 0, st_>>>(d_, stage_.dev(base), n);
        PK_CUDA(cudaGetLastError());
        PK_CUDA(stage_.commit(st_));
        return 0;
    }

    int kill_world(const int *slots, int n, int world) override
    {
        Dev<T> d = d_;
        d.man_old = man_[parity_];
        if (n > 0)
        {
            int *ds;
            PK_CUDA(cudaMallocAsync(&ds, sizeof(int) * size_t(n), st_));
            PK_CUDA(cudaMemcpyAsync(ds, slots, sizeof(int) * size_t(n), cudaMemcpyHostToDevice, st_));
            k_kill_bodies<T><<<grid(n), 256, 0, st_>>>(d, ds, n);
            PK_CUDA(cudaFreeAsync(ds, st_));
        }
        k_purge_world<T><<<grid(cfg_.pair_cap), 256, 0, st_>>>(d, uint32_t(world));
        PK_CUDA(cudaGetLastError());
        PK_CUDA(cudaStreamSynchronize(st_));
        return 0;
    }

    int set_active_mask(const uint8_t *mask, int n) override
    {
        if (n != cfg_.max_worlds) return -3;
        if (!mask_dev_) PK_CUDA(cudaMalloc(&mask_dev_, size_t(cfg_.max_worlds)));
        PK_CUDA(cudaMemcpyAsync(mask_dev_, mask, size_t(n), cudaMemcpyHostToDevice, st_));
        k_set_active<T><<<grid(n), 256, 0, st_>>>(d_, mask_dev_, n);
        PK_CUDA(cudaGetLastError());
        return 0;
    }

    int kill_body(int slot, int world, int local) override
    {
        k_kill_body<T><<<1, 1, 0, st_>>>(d_, slot);
        Dev<T> d = d_;
        d.man_old = man_[parity_];
        k_purge_pairs<T><<<grid(cfg_.pair_cap), 256, 0, st_>>>(d, uint32_t(world), uint32_t(local));
        PK_CUDA(cudaGetLastError());
        PK_CUDA(cudaStreamSynchronize(st_));
        return 0;
    }

    int step(double dt) override
    {
        int rc = enqueue_step(T(dt), parity_);
        if (rc) return rc;
        parity_ ^= 1;
        return 0;
    }

    // Captures the step of each parity. A graph of the same shape as the one instantiated (the
    // usual case when worlds are admitted or retired: the same launches with other grid sizes or
    // arguments) updates the executable graph in place, which costs a fraction of instantiating.
    int capture_graph(double dt) override
    {
        for (int k = 0; k < 2; ++k)
        {
            cudaGraph_t g;
            PK_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
            capturing_ = true;
            int rc = enqueue_step(T(dt), k);
            capturing_ = false;
            cudaError_t e = cudaStreamEndCapture(st_, &g);
            if (rc)
            {
                if (e == cudaSuccess) cudaGraphDestroy(g);
                return rc;
            }
            PK_CUDA(e);
            if (graph_exec_[k])
            {
                cudaGraphExecUpdateResultInfo info;
                if (cudaGraphExecUpdate(graph_exec_[k], g, &info) != cudaSuccess)
                {
                    (void)cudaGetLastError(); // not updatable (another shape): instantiate anew
                    cudaGraphExecDestroy(graph_exec_[k]);
                    graph_exec_[k] = nullptr;
                }
            }
            if (!graph_exec_[k])
            {
                cudaError_t ie = cudaGraphInstantiate(&graph_exec_[k], g, 0);
                if (ie != cudaSuccess)
                {
                    cudaGraphDestroy(g);
                    graph_exec_[k] = nullptr;
                    PK_CUDA(ie);
                }
            }
            cudaGraphDestroy(g);
        }
        return 0;
    }

    int launch_graph() override
    {
        if (!graph_exec_[parity_]) return -2;
        PK_CUDA(cudaGraphLaunch(graph_exec_[parity_], st_));
        parity_ ^= 1;
        return 0;
    }

    int set_timing(int enable) override
    {
        timing_ = enable != 0;
        return 0;
    }

    int read_stage_times(double *ms, int *count) override
    {
        PK_CUDA(cudaStreamSynchronize(st_));
        PK_CUDA(accumulate_stage_times());
        for (int k = 0; k < kStageRows; ++k)
        {
            ms[k] = stage_ms_[k];
            count[k] = stage_n_[k];
            stage_ms_[k] = 0.0;
            stage_n_[k] = 0;
        }
        return kStageRows;
    }

    int synchronize(StepCounters *c) override
    {
        PK_CUDA(cudaStreamSynchronize(st_));
        PK_CUDA(cudaStreamSynchronize(cs_)); // read-backs in flight
        PK_CUDA(cudaGetLastError());
        PK_CUDA(accumulate_stage_times());
        int h[32];
        PK_CUDA(cudaMemcpy(h, counters_, sizeof(h), cudaMemcpyDeviceToHost));
        if (c)
        {
            c->nleaf = h[1];
            c->npairs = h[2];
            c->status = h[4];
            c->launches = launches_;
            c->gjk = h[6] + h[8];
            c->gjk_heavy = h[8];
            c->epa = h[7] + h[9];
            c->epa_heavy = h[9];
            unsigned long long it[3];
            std::memcpy(it, h + 10, sizeof(it));
            c->gjk_iters = (long long)it[0];
            c->epa_iters = (long long)it[1];
            c->epa_iters_heavy = (long long)it[2];
            unsigned long long sv;
            std::memcpy(&sv, h + 24, sizeof(sv));
            c->support_verts = (long long)sv;
        }
        int zero = 0;
        PK_CUDA(cudaMemcpy(counters_ + 4, &zero, sizeof(int), cudaMemcpyHostToDevice));
        return 0;
    }

    // The state rows are packed on the device (k_pack_bodies) and copied to the caller's buffer in
    // one transfer; a buffer pinned with pk_host_register takes the direct path.
    cudaError_t ensure_pack(int n)
    {
        if (size_t(n) <= pack_cap_) return cudaSuccess;
        // the copies in flight read the old buffers
        cudaError_t e = cudaStreamSynchronize(cs_);
        if (e != cudaSuccess) return e;
        for (int k = 0; k < 2; ++k)
        {
            if (pack_[k]) cudaFree(pack_[k]);
            pack_[k] = nullptr;
        }
        pack_cap_ = 0;
        for (int k = 0; k < 2; ++k)
            if ((e = cudaMalloc(&pack_[k], sizeof(double) * 14 * size_t(n))) != cudaSuccess) return e;
        pack_cap_ = size_t(n);
        return cudaSuccess;
    }

    int read_bodies(double *out, int n) override
    {
        if (n > nslots_) n = nslots_;
        if (n <= 0) return 0;
        PK_CUDA(ensure_pack(n));
        PK_CUDA(cudaStreamSynchronize(cs_)); // buffer 0 may still be in a read-back's copy
        k_pack_bodies<T><<<grid(n), 256, 0, st_>>>(d_, pack_[0], n);
        PK_CUDA(cudaGetLastError());
        PK_CUDA(cudaMemcpyAsync(out, pack_[0], sizeof(double) * 14 * size_t(n), cudaMemcpyDeviceToHost, st_));
        PK_CUDA(cudaStreamSynchronize(st_));
        return n;
    }

    // Double-buffered: the rows of this call are packed into one buffer on the world's stream
    // (after the steps enqueued so far, before the next ones) and copied out on the copy stream,
    // while the next step runs; a buffer is packed again only after its previous copy has ended.
    int read_bodies_async(double *out, int n) override
    {
        if (n > nslots_) n = nslots_;
        if (n <= 0) return 0;
        PK_CUDA(ensure_pack(n));
        const int b = pack_next_;
        pack_next_ ^= 1;
        PK_CUDA(cudaStreamWaitEvent(st_, copied_[b], 0));
        k_pack_bodies<T><<<grid(n), 256, 0, st_>>>(d_, pack_[b], n);
        PK_CUDA(cudaGetLastError());
        PK_CUDA(cudaEventRecord(packed_[b], st_));
        PK_CUDA(cudaStreamWaitEvent(cs_, packed_[b], 0));
        PK_CUDA(cudaMemcpyAsync(out, pack_[b], sizeof(double) * 14 * size_t(n), cudaMemcpyDeviceToHost, cs_));
        PK_CUDA(cudaEventRecord(copied_[b], cs_));
        return n;
    }

    int write_state(int slot, const double *s) override
    {
        Pose<T> p;
        Vel<T> v;
        for (int k = 0; k < 3; ++k)
        {
            p.p[k] = T(s[k]);
            v.v[k] = T(s[7 + k]);
            v.w[k] = T(s[10 + k]);
        }
        for (int k = 0; k < 4; ++k) p.q[k] = T(s[3 + k]);
        PK_CUDA(cudaMemcpy(d_.pose + slot, &p, sizeof(p), cudaMemcpyHostToDevice));
        PK_CUDA(cudaMemcpy(d_.vel + slot, &v, sizeof(v), cudaMemcpyHostToDevice));
        k_refresh_derived<T><<<1, 32, 0, st_>>>(d_, slot, 1);
        PK_CUDA(cudaGetLastError());
        PK_CUDA(cudaStreamSynchronize(st_));
        return 0;
    }

    int read_pairs(uint64_t *keys, uint64_t *slots, int cap) override
    {
        int np = 0;
        PK_CUDA(cudaStreamSynchronize(st_));
        PK_CUDA(cudaMemcpy(&np, d_.npairs_old, sizeof(int), cudaMemcpyDeviceToHost));
        int n = np < cap ? np : cap;
        if (n > 0 && keys) PK_CUDA(cudaMemcpy(keys, d_.key_old, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost));
        if (n > 0 && slots && last_sval_) PK_CUDA(cudaMemcpy(slots, last_sval_, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost));
        return np;
    }

    int read_manifolds(uint64_t *keys, int *counts, double *contacts, int cap) override
    {
        int np = 0;
        PK_CUDA(cudaStreamSynchronize(st_));
        PK_CUDA(cudaMemcpy(&np, d_.npairs_old, sizeof(int), cudaMemcpyDeviceToHost));
        int n = np < cap ? np : cap;
        if (n > 0)
        {
            std::vector<Manifold<T>> m(n);
            PK_CUDA(cudaMemcpy(m.data(), man_[parity_], sizeof(Manifold<T>) * n, cudaMemcpyDeviceToHost));
            if (keys) PK_CUDA(cudaMemcpy(keys, d_.key_old, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost));
            for (int i = 0; i < n; ++i)
            {
                if (counts) counts[i] = m[i].n;
                if (!contacts) continue;
                for (int k = 0; k < 4; ++k)
                {
                    double *o = contacts + (size_t(i) * 4 + k) * 13;
                    const Contact<T> &c = m[i].c[k];
                    if (k >= m[i].n)
                    {
                        for (int z = 0; z < 13; ++z) o[z] = 0.0;
                        continue;
                    }
                    for (int z = 0; z < 3; ++z)
                    {
                        o[z] = double(c.n[z]);
                        o[3 + z] = double(c.la[z]);
                        o[6 + z] = double(c.lb[z]);
                    }
                    o[9] = double(c.depth);
                    o[10] = c.imp[0];
                    o[11] = c.imp[1];
                    o[12] = c.imp[2];
                }
            }
        }
        return np;
    }

    int read_events(uint64_t *keys, int *kinds, int cap) override
    {
        int np = 0;
        PK_CUDA(cudaStreamSynchronize(st_));
        PK_CUDA(cudaMemcpy(&np, d_.npairs_old, sizeof(int), cudaMemcpyDeviceToHost));
        if (np == 0) return 0;
        std::vector<uint8_t> ev(np);
        std::vector<uint64_t> k(np);
        PK_CUDA(cudaMemcpy(ev.data(), d_.event, np, cudaMemcpyDeviceToHost));
        PK_CUDA(cudaMemcpy(k.data(), d_.key_old, sizeof(uint64_t) * np, cudaMemcpyDeviceToHost));
        int cnt = 0;
        for (int i = 0; i < np; ++i)
        {
            if (!ev[i]) continue;
            if (cnt < cap)
            {
                if (keys) keys[cnt] = k[i];
                if (kinds) kinds[cnt] = ev[i];
            }
            ++cnt;
        }
        return cnt;
    }

    int read_colours(uint64_t *keys, int *colours, int cap, int *nc0) override
    {
        int np = 0;
        PK_CUDA(cudaStreamSynchronize(st_));
        PK_CUDA(cudaMemcpy(&np, d_.npairs_old, sizeof(int), cudaMemcpyDeviceToHost));
        std::vector<int> col(np > 0 ? np : 1);
        std::vector<uint64_t> k(np > 0 ? np : 1);
        if (np > 0)
        {
            PK_CUDA(cudaMemcpy(col.data(), d_.pair_colour, sizeof(int) * np, cudaMemcpyDeviceToHost));
            PK_CUDA(cudaMemcpy(k.data(), d_.key_old, sizeof(uint64_t) * np, cudaMemcpyDeviceToHost));
            // the solver colours only pairs with contact rows; the others read -2
            std::vector<uint8_t> mask(static_cast<size_t>(np));
            PK_CUDA(cudaMemcpy(mask.data(), d_.rowmask, size_t(np), cudaMemcpyDeviceToHost));
            for (int i = 0; i < np; ++i)
                if (!mask[i]) col[i] = -2;
        }
        if (nc0) PK_CUDA(cudaMemcpy(nc0, d_.ncolours, sizeof(int), cudaMemcpyDeviceToHost));
        int cnt = 0;
        for (int i = 0; i < np; ++i)
        {
            if (col[i] < 0) continue;
            if (cnt < cap)
            {
                if (keys) keys[cnt] = k[i];
                if (colours) colours[cnt] = col[i];
            }
            ++cnt;
        }
        return cnt;
    }

    int collide(const void *specs_a, const void *specs_b, int n, double *out, int *hit, int *status) override
    {
        if (n <= 0) return 0;
        ShapeSpec *da, *db;
        double *dout;
        int *dhit, *dst;
        PK_CUDA(cudaMalloc(&da, sizeof(ShapeSpec) * n));
        PK_CUDA(cudaMalloc(&db, sizeof(ShapeSpec) * n));
        PK_CUDA(cudaMalloc(&dout, sizeof(double) * 10 * n));
        PK_CUDA(cudaMalloc(&dhit, sizeof(int) * n));
        PK_CUDA(cudaMalloc(&dst, sizeof(int) * n));
        PK_CUDA(cudaMemcpy(da, specs_a, sizeof(ShapeSpec) * n, cudaMemcpyHostToDevice));
        PK_CUDA(cudaMemcpy(db, specs_b, sizeof(ShapeSpec) * n, cudaMemcpyHostToDevice));
        PK_CUDA(cudaMemset(dout, 0, sizeof(double) * 10 * n));
        k_collide_batch<T><<<(n + 127) / 128, 128, 0, st_>>>(da, db, n, d_.verts, shape_range_, d_.clusters,
                                                              shape_rmax_, dout, dhit, dst, nullptr);
        PK_CUDA(cudaGetLastError());
        PK_CUDA(cudaStreamSynchronize(st_));
        PK_CUDA(cudaMemcpy(out, dout, sizeof(double) * 10 * n, cudaMemcpyDeviceToHost));
        PK_CUDA(cudaMemcpy(hit, dhit, sizeof(int) * n, cudaMemcpyDeviceToHost));
        PK_CUDA(cudaMemcpy(status, dst, sizeof(int) * n, cudaMemcpyDeviceToHost));
        cudaFree(da);
        cudaFree(db);
        cudaFree(dout);
        cudaFree(dhit);
        cudaFree(dst);
        return 0;
    }

    // World raycast: rebuild the LBVH over every alive body of every world (the step's tree covers
    // only the worlds that stepped, and bodies may have changed since), then one thread per ray.
    int raycast(const double *rays, int n, int cap, int *counts, int *slots, double *dists) override
    {
        if (n <= 0) return 0;
        Dev<T> d = d_;
        d.mkey = mkey_[0];
        d.mval = mval_[0];
        const int N = cfg_.body_cap;
        const int gb = grid(N);
        k_tree_reset<T><<<grid(cfg_.max_worlds), 256, 0, st_>>>(d);
        k_morton<T><<<gb, 256, 0, st_>>>(d, true);
        bool in1 = radix_sort<uint64_t>(mkey_[0], mval_[0], mkey_[1], mval_[1], d.nleaf, cfg_.wbits + 31,
                                        cfg_.sort_blocks_bodies, hist_, st_);
        const uint64_t *skey = in1 ? mkey_[1] : mkey_[0];
        const uint64_t *sval = in1 ? mval_[1] : mval_[0];
        k_lbvh_build<T><<<gb, 256, 0, st_>>>(d, skey);
        k_zero_ints<<<gb, 256, 0, st_>>>(d.refit_flag, N);
        k_lbvh_refit<T><<<gb, 256, 0, st_>>>(d, sval);
        double *drays = nullptr;
        int *dcnt = nullptr, *dslot = nullptr;
        T *dt = nullptr;
        const size_t m = size_t(n) * size_t(cap);
        PK_CUDA(cudaMalloc(&drays, sizeof(double) * 8 * size_t(n)));
        PK_CUDA(cudaMalloc(&dcnt, sizeof(int) * size_t(n)));
        PK_CUDA(cudaMalloc(&dslot, sizeof(int) * m));
        PK_CUDA(cudaMalloc(&dt, sizeof(T) * m));
        PK_CUDA(cudaMemcpyAsync(drays, rays, sizeof(double) * 8 * size_t(n), cudaMemcpyHostToDevice, st_));
        k_raycast<T><<<(n + 127) / 128, 128, 0, st_>>>(d, sval, drays, n, cap, dcnt, dslot, dt);
        PK_CUDA(cudaGetLastError());
        PK_CUDA(cudaStreamSynchronize(st_));
        std::vector<T> ht(m);
        PK_CUDA(cudaMemcpy(counts, dcnt, sizeof(int) * size_t(n), cudaMemcpyDeviceToHost));
        PK_CUDA(cudaMemcpy(slots, dslot, sizeof(int) * m, cudaMemcpyDeviceToHost));
        PK_CUDA(cudaMemcpy(ht.data(), dt, sizeof(T) * m, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < m; ++i) dists[i] = double(ht[i]);
        cudaFree(drays);
        cudaFree(dcnt);
        cudaFree(dslot);
        cudaFree(dt);
        return 0;
    }

    int set_triangles(const std::vector<int> &tris, const std::vector<int> &range) override
    {
        const size_t nt = tris.size(), ns = range.size() / 2;
        if (nt > tri_cap_)
        {
            if (tris_) cudaFree(tris_);
            tris_ = nullptr;
            tri_cap_ = nt + nt / 2 + 64;
            PK_CUDA(cudaMalloc(&tris_, sizeof(int) * tri_cap_));
        }
        if (ns > trange_cap_)
        {
            if (trange_) cudaFree(trange_);
            trange_ = nullptr;
            trange_cap_ = ns + ns / 2 + 16;
            PK_CUDA(cudaMalloc(&trange_, sizeof(int2) * trange_cap_));
        }
        if (nt) PK_CUDA(cudaMemcpyAsync(tris_, tris.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, st_));
        if (ns) PK_CUDA(cudaMemcpyAsync(trange_, range.data(), sizeof(int2) * ns, cudaMemcpyHostToDevice, st_));
        PK_CUDA(cudaStreamSynchronize(st_));
        return 0;
    }

    int mesh_raycast(const MeshRayIn *rays, int n, MeshHitOut *out) override
    {
        if (n <= 0) return 0;
        MeshRayIn *dr = nullptr;
        MeshHitOut *dh = nullptr;
        PK_CUDA(cudaMalloc(&dr, sizeof(MeshRayIn) * size_t(n)));
        PK_CUDA(cudaMalloc(&dh, sizeof(MeshHitOut) * size_t(n)));
        PK_CUDA(cudaMemcpyAsync(dr, rays, sizeof(MeshRayIn) * size_t(n), cudaMemcpyHostToDevice, st_));
        k_mesh_raycast<T><<<(n + 127) / 128, 128, 0, st_>>>(d_, tris_, trange_, dr, n, dh);
        PK_CUDA(cudaGetLastError());
        PK_CUDA(cudaMemcpyAsync(out, dh, sizeof(MeshHitOut) * size_t(n), cudaMemcpyDeviceToHost, st_));
        PK_CUDA(cudaStreamSynchronize(st_));
        cudaFree(dr);
        cudaFree(dh);
        return 0;
    }

    // Joints, ordered by (world, type, arena slot): 5 ints (type, slot a, slot b, local a, local b)
    // and 25 doubles (la3 lb3 axa3 axb3 va3 wa3 qrel4 distance stiffness damping) each, their
    // accumulated impulses (6 each) and every world's range. Growing the buffers drops a captured
    // step graph (its kernels hold the old pointers).
    int set_joints(const int *ints, const double *params, const double *acc, int n, const int *jstart,
                   const int *jend) override
    {
        PK_CUDA(cudaStreamSynchronize(st_));
        if (n > joint_cap_)
        {
            int cap = n < 64 ? 64 : n;
            void *old[] = {const_cast<JointDev<T> *>(d_.joints), d_.jrows, d_.jnrows, d_.jacc};
            for (void *p : old)
                if (p) cudaFree(p);
            JointDev<T> *jd;
            PK_CUDA(alloc(&jd, size_t(cap)));
            d_.joints = jd;
            PK_CUDA(alloc(&d_.jrows, size_t(cap) * kJointMaxRows));
            PK_CUDA(alloc(&d_.jnrows, size_t(cap)));
            PK_CUDA(alloc(&d_.jacc, size_t(cap) * kJointMaxRows));
            PK_CUDA(cudaMemset(d_.jnrows, 0, sizeof(int) * size_t(cap)));
            joint_cap_ = cap;
            for (int k = 0; k < 2; ++k)
            {
                if (graph_exec_[k]) cudaGraphExecDestroy(graph_exec_[k]);
                graph_exec_[k] = nullptr;
            }
        }
        std::vector<JointDev<T>> h(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i)
        {
            JointDev<T> &j = h[size_t(i)];
            const int *ii = ints + 5 * size_t(i);
            const double *p = params + 25 * size_t(i);
            j.type = ii[0];
            j.a = ii[1];
            j.b = ii[2];
            j.local_a = ii[3];
            j.local_b = ii[4];
            j.pad[0] = j.pad[1] = j.pad[2] = 0;
            for (int k = 0; k < 3; ++k)
            {
                j.la[k] = T(p[k]);
                j.lb[k] = T(p[3 + k]);
                j.axa[k] = T(p[6 + k]);
                j.axb[k] = T(p[9 + k]);
                j.va[k] = T(p[12 + k]);
                j.wa[k] = T(p[15 + k]);
            }
            for (int k = 0; k < 4; ++k) j.qrel[k] = T(p[18 + k]);
            j.distance = T(p[22]);
            j.stiffness = T(p[23]);
            j.damping = T(p[24]);
        }
        if (n > 0)
        {
            PK_CUDA(cudaMemcpy(const_cast<JointDev<T> *>(d_.joints), h.data(), sizeof(JointDev<T>) * size_t(n),
                               cudaMemcpyHostToDevice));
            PK_CUDA(cudaMemcpy(d_.jacc, acc, sizeof(double) * kJointMaxRows * size_t(n), cudaMemcpyHostToDevice));
        }
        PK_CUDA(cudaMemcpy(d_.jstart, jstart, sizeof(int) * cfg_.max_worlds, cudaMemcpyHostToDevice));
        PK_CUDA(cudaMemcpy(d_.jend, jend, sizeof(int) * cfg_.max_worlds, cudaMemcpyHostToDevice));
        PK_CUDA(cudaMemcpy(counters_ + 17, &n, sizeof(int), cudaMemcpyHostToDevice));
        njoints_ = n;
        return 0;
    }

    int read_joint_acc(double *acc, int n) override
    {
        PK_CUDA(cudaStreamSynchronize(st_));
        if (n > 0) PK_CUDA(cudaMemcpy(acc, d_.jacc, sizeof(double) * kJointMaxRows * size_t(n), cudaMemcpyDeviceToHost));
        return 0;
    }

    int read_pose(int slot, double *out7) override
    {
        Pose<T> p;
        PK_CUDA(cudaStreamSynchronize(st_));
        PK_CUDA(cudaMemcpy(&p, d_.pose + slot, sizeof(p), cudaMemcpyDeviceToHost));
        for (int k = 0; k < 3; ++k) out7[k] = double(p.p[k]);
        for (int k = 0; k < 4; ++k) out7[3 + k] = double(p.q[k]);
        return 0;
    }

    int collide_device(const void *specs_a, const void *specs_b, int n, double *out, int *hit, int *status,
                       int *status_any) override
    {
        if (n <= 0) return 0;
        k_collide_batch<T><<<(n + 127) / 128, 128, 0, st_>>>(static_cast<const ShapeSpec *>(specs_a),
                                                              static_cast<const ShapeSpec *>(specs_b), n, d_.verts,
                                                              shape_range_, d_.clusters, shape_rmax_, out, hit, status,
                                                              status_any);
        PK_CUDA(cudaGetLastError());
        return 0;
    }

private:
    EngineConfig cfg_{};
    Dev<T> d_{};
    cudaStream_t st_ = nullptr;
    cudaStream_t st2_ = nullptr; // the solver's small-world launches run beside the large-world one
    cudaStream_t st3_ = nullptr; // with st2_: the sweep's size classes run side by side
    cudaEvent_t fork_ = nullptr, join_ = nullptr, join3_ = nullptr;
    int sms_ = 1;
    int nslots_ = 0;
    int parity_ = 0;
    int last_err_ = 0;
    int *counters_ = nullptr;
    uint64_t *mkey_[2] = {nullptr, nullptr}, *mval_[2] = {nullptr, nullptr};
    uint64_t *pkey_[2] = {nullptr, nullptr}, *pval_[2] = {nullptr, nullptr};
    Manifold<T> *man_[2] = {nullptr, nullptr};
    uint64_t *last_sval_ = nullptr;
    uint32_t *hist_ = nullptr;
    ShapeRange *shape_range_ = nullptr;
    Aabb<T> *shape_box_ = nullptr;
    T *shape_rmax_ = nullptr;
    T *clusters_ = nullptr;
    size_t clusters_cap_ = 0;
    cudaGraphExec_t graph_exec_[2] = {nullptr, nullptr};
    int joint_cap_ = 0, njoints_ = 0;
    static constexpr size_t kMaxSolveSmem = 160 * 1024;
    // the FP64 form's solver sweeps are long FP64 chains: small worlds share CTAs (solve groups)
    Tunables tune_ = sizeof(T) == 8 ? Tunables{256, 512, 2, 128, 256, 1024, 128, 0} : Tunables{};
    int big_worlds_ = 0;
    std::vector<int> goff_; // solve groups: first index in the world order of each group, then the end
    int *goff_dev_ = nullptr;
    int group_cache_ = 0; // the largest group's local indices (its velocity cache)
    int big_cache_ = 0;
    size_t big_smem_ = 0; // dynamic shared memory of the large-world launch
    double *pack_[2] = {nullptr, nullptr}; // read-back staging: 14 doubles per slot, double-buffered
    size_t pack_cap_ = 0;
    int pack_next_ = 0;
    cudaStream_t cs_ = nullptr; // read-back copies
    cudaEvent_t packed_[2] = {nullptr, nullptr}, copied_[2] = {nullptr, nullptr};
    std::vector<int> order_, nlocal_;
    std::vector<int> grid_worlds_;             // worlds solved by the cooperative grid solver
    static constexpr int kGridWorld = 16384;   // local indices above which a world leaves the CTA solver
    GridScratch *grid_scratch_ = nullptr;
    int grid_blocks_ = 1;
    bool timing_ = false;
    bool capturing_ = false;
    uint8_t *mask_dev_ = nullptr;
    int *tris_ = nullptr;   // triangles of every shape (mesh ray queries)
    int2 *trange_ = nullptr;
    size_t tri_cap_ = 0, trange_cap_ = 0;
    StagingRing stage_; // pinned staging of the asynchronous uploads (allocated on first use)
    cudaError_t ensure_staging() { return stage_.ready() ? cudaSuccess : stage_.init(size_t(64) << 20); }
    int launches_ = 0;
    // per timed step: the kStages + 1 stage boundaries, then three marks inside the narrowphase
    static constexpr int kMarks = kStages + 4;
    std::vector<cudaEvent_t> events_;
    int timed_steps_ = 0;
    double stage_ms_[kStageRows] = {};
    int stage_n_[kStageRows] = {};

    cudaError_t mark(int stage)
    {
        if (!timing_ || capturing_) return cudaSuccess;
        size_t idx = size_t(timed_steps_) * kMarks + size_t(stage);
        while (events_.size() <= idx)
        {
            cudaEvent_t e;
            cudaError_t err = cudaEventCreate(&e);
            if (err != cudaSuccess) return err;
            events_.push_back(e);
        }
        return cudaEventRecord(events_[idx], st_);
    }
    cudaError_t accumulate_stage_times()
    {
        // rows: stage k spans marks k..k+1; the narrowphase's parts span 5..10, 10..11, 11..12, 12..6
        const int from[kStageRows] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 5, kStages + 1, kStages + 2, kStages + 3};
        const int to[kStageRows] = {1, 2, 3, 4, 5, 6, 7, 8, 9, kStages + 1, kStages + 2, kStages + 3, 6};
        for (int s = 0; s < timed_steps_; ++s)
            for (int k = 0; k < kStageRows; ++k)
            {
                float ms = 0.f;
                cudaError_t e = cudaEventElapsedTime(&ms, events_[size_t(s) * kMarks + from[k]],
                                                     events_[size_t(s) * kMarks + to[k]]);
                if (e != cudaSuccess) return e;
                stage_ms_[k] += ms;
                stage_n_[k] += 1;
            }
        timed_steps_ = 0;
        return cudaSuccess;
    }

    template <class U> cudaError_t alloc(U **p, size_t n)
    {
        if (n == 0) n = 1;
        return cudaMalloc(reinterpret_cast<void **>(p), sizeof(U) * n);
    }
    template <class U> cudaError_t alloc(const U **p, size_t n)
    {
        if (n == 0) n = 1;
        return cudaMalloc(const_cast<void **>(reinterpret_cast<const void **>(p)), sizeof(U) * n);
    }
    static int solve_threads(int t) { return t < solve_max_threads<T>() ? t : solve_max_threads<T>(); }
    template <int C> void launch_broad(const Dev<T> &d, const uint64_t *skey, const uint64_t *sval, cudaStream_t st)
    {
        constexpr BroadClass c = kBroadClasses[C];
        k_broad_small<T, c.minn, c.maxn, c.qcap, c.threads>
            <<<cfg_.max_worlds, c.threads, broad_smem_bytes<c.maxn, c.qcap>(), st>>>(d, skey, sval);
    }
    // The joint-free instances serve batches that never had joints (buffers unallocated).
    void launch_solve(int blocks, int threads, size_t smem, const Dev<T> &d, const uint64_t *pv, int first, int cache,
                      cudaStream_t st)
    {
        threads = solve_threads(threads);
        const bool joints = joint_cap_ > 0;
        if (threads > 256 && joints)
            k_solve_world<T, solve_max_threads<T>(), true><<<blocks, threads, smem, st>>>(d, pv, first, cache, kGridWorld);
        else if (threads > 256)
            k_solve_world<T, solve_max_threads<T>(), false><<<blocks, threads, smem, st>>>(d, pv, first, cache, kGridWorld);
        else if (joints)
            k_solve_world<T, 256, true><<<blocks, threads, smem, st>>>(d, pv, first, cache, kGridWorld);
        else
            k_solve_world<T, 256, false><<<blocks, threads, smem, st>>>(d, pv, first, cache, kGridWorld);
    }
    int grid(int n) const
    {
        int g = (n + 255) / 256;
        int cap = sms_ * 8;
        if (g > cap) g = cap;
        return g < 1 ? 1 : g;
    }
    void release()
    {
        for (int k = 0; k < 2; ++k)
            if (graph_exec_[k]) cudaGraphExecDestroy(graph_exec_[k]);
        void *ps[] = {d_.pose, d_.vel, d_.iw, d_.iwinv, d_.prm, d_.tbox, d_.meta, counters_, d_.wp, d_.wbounds,
                      d_.wroot, d_.wleaf_lo, d_.wleaf_hi, d_.wlive, d_.mstart, d_.mend, d_.mstart_old, d_.mend_old, d_.nstart, d_.nend, d_.jstart, d_.jend,
                      const_cast<JointDev<T> *>(d_.joints), d_.jrows, d_.jnrows, d_.jacc, d_.ncolours, mkey_[0], mkey_[1], mval_[0], mval_[1],
                      pkey_[0], pkey_[1], pval_[0], pval_[1], man_[0], man_[1], d_.nodes, d_.parent,
                      d_.leaf_parent, d_.refit_flag, d_.key_old, d_.val_old, d_.event, d_.old_idx, d_.gjk_list, d_.clist, d_.gjk_list2, d_.gcls,
                      d_.epa_list, d_.epa_simplex, d_.rowidx, d_.rows, d_.racc, d_.raccf, d_.rdel, d_.rowmask, d_.colour, d_.colour_tmp, d_.pair_colour,
                      d_.order, d_.srec, d_.crec, d_.owner, d_.used, const_cast<int *>(d_.world_order), goff_dev_,
                      const_cast<int *>(d_.world_nlocal), hist_, const_cast<T *>(d_.verts), const_cast<float *>(d_.verts32),
                      const_cast<float *>(d_.shape32), d_.pose32, shape_range_, shape_box_,
                      shape_rmax_, clusters_, mask_dev_, grid_scratch_};
        for (void *p : ps)
            if (p) cudaFree(p);
        if (cs_) cudaStreamSynchronize(cs_);
        for (int k = 0; k < 2; ++k)
        {
            if (pack_[k]) cudaFree(pack_[k]);
            pack_[k] = nullptr;
            if (packed_[k]) cudaEventDestroy(packed_[k]);
            if (copied_[k]) cudaEventDestroy(copied_[k]);
            packed_[k] = copied_[k] = nullptr;
        }
        pack_cap_ = 0;
        if (cs_) cudaStreamDestroy(cs_);
        cs_ = nullptr;
        stage_.release();
        if (tris_) cudaFree(tris_);
        if (trange_) cudaFree(trange_);
        tris_ = nullptr;
        trange_ = nullptr;
        for (cudaEvent_t e : events_) cudaEventDestroy(e);
        if (st_) cudaStreamDestroy(st_);
        st_ = nullptr;
        if (st2_) cudaStreamDestroy(st2_);
        st2_ = nullptr;
        if (st3_) cudaStreamDestroy(st3_);
        st3_ = nullptr;
        if (fork_) cudaEventDestroy(fork_);
        if (join_) cudaEventDestroy(join_);
        if (join3_) cudaEventDestroy(join3_);
        fork_ = join_ = join3_ = nullptr;
    }

    int enqueue_step(T dt, int parity)
    {
        Dev<T> d = d_;
        d.man_old = man_[parity];
        d.man_new = man_[parity ^ 1];
        d.mkey = mkey_[0]; // Morton keys are written here, the radix sort ping-pongs with [1]
        d.mval = mval_[0];
        d.pkey = pkey_[0]; // pairs are emitted here, the radix sort ping-pongs with [1]
        d.pval = pval_[0];
        const int N = cfg_.body_cap;
        const int gb = grid(N);
        const int gp = grid(cfg_.pair_cap);
        const int mpasses = (cfg_.wbits + 31 + 7) / 8, ppasses = (cfg_.wbits + 2 * cfg_.lbits + 7) / 8;
        launches_ = 26 + int(grid_worlds_.size()) + (big_worlds_ > 0) + (cfg_.max_worlds > big_worlds_) + 3 * mpasses + 3 * ppasses;
        PK_CUDA(mark(0));
        k_begin_step<T><<<grid(cfg_.max_worlds), 256, 0, st_>>>(d);
        k_integrate_vel<T><<<gb, 256, 0, st_>>>(d, dt);
        PK_CUDA(mark(1));
        k_morton<T><<<gb, 256, 0, st_>>>(d, false);
        // sort the bodies of active worlds by (world, static, Morton); the two lowest digits, Morton
        // bits only the LBVH needs, are skipped in steps where no world traverses
        bool in1 = radix_sort<uint64_t>(mkey_[0], mval_[0], mkey_[1], mval_[1], d.nleaf, cfg_.wbits + 31,
                                        cfg_.sort_blocks_bodies, hist_, st_, d.all_small, 2);
        const uint64_t *skey = in1 ? mkey_[1] : mkey_[0];
        const uint64_t *sval = in1 ? mval_[1] : mval_[0];
        PK_CUDA(mark(2));
        k_lbvh_build<T><<<gb, 256, 0, st_>>>(d, skey, true);
        k_zero_ints<<<gb, 256, 0, st_>>>(d.refit_flag, N);
        k_lbvh_refit<T><<<gb, 256, 0, st_>>>(d, sval, true);
        PK_CUDA(mark(3));
        k_traverse<T><<<(N + tune_.traverse_threads - 1) / tune_.traverse_threads, tune_.traverse_threads, 0, st_>>>(d, sval);
        // The sweep's three size classes run side by side, so that the SMs one class's last wave
        // leaves idle take the others' CTAs. Their worlds are disjoint, and the pair list they
        // append to is sorted after them.
        PK_CUDA(cudaEventRecord(fork_, st_));
        PK_CUDA(cudaStreamWaitEvent(st2_, fork_, 0));
        PK_CUDA(cudaStreamWaitEvent(st3_, fork_, 0));
        launch_broad<2>(d, skey, sval, st_);
        launch_broad<1>(d, skey, sval, st2_);
        launch_broad<0>(d, skey, sval, st3_);
        PK_CUDA(cudaEventRecord(join_, st2_));
        PK_CUDA(cudaEventRecord(join3_, st3_));
        PK_CUDA(cudaStreamWaitEvent(st_, join_, 0));
        PK_CUDA(cudaStreamWaitEvent(st_, join3_, 0));
        k_clamp_pairs<T><<<1, 1, 0, st_>>>(d);
        k_kept_count<T><<<cfg_.max_worlds, 256, 0, st_>>>(d);
        PK_CUDA(mark(4));
        // sort the new pairs, then assemble every world's segment (new pairs of active worlds,
        // kept pairs of idle ones) in world order into the sort's other buffer
        bool p1 = radix_sort<uint64_t>(pkey_[0], pval_[0], pkey_[1], pval_[1], d.npairs,
                                       cfg_.wbits + 2 * cfg_.lbits, cfg_.sort_blocks_pairs, hist_, st_);
        const uint64_t *nk = p1 ? pkey_[1] : pkey_[0];
        const uint64_t *nv = p1 ? pval_[1] : pval_[0];
        uint64_t *ak = p1 ? pkey_[0] : pkey_[1];
        uint64_t *av = p1 ? pval_[0] : pval_[1];
        k_pair_bounds<T><<<gp, 256, 0, st_>>>(d, nk);
        k_pair_segments<T><<<1, 1024, 0, st_>>>(d);
        k_assemble_new<T><<<gp, 256, 0, st_>>>(d, nk, nv, ak, av);
        k_assemble_kept<T><<<cfg_.max_worlds, 256, 0, st_>>>(d, ak, av);
        const uint64_t *pk = ak;
        const uint64_t *pv = av;
        last_sval_ = av;
        PK_CUDA(mark(5));
        k_old_index<T><<<gp, 256, 0, st_>>>(d, pk);
        k_narrow_pre<T><<<gp, 256, 0, st_>>>(d, pk, pv);
        PK_CUDA(mark(kStages + 1));
        k_narrow_axis<T><<<grid(cfg_.pair_cap) * 2, 128, 0, st_>>>(d, pv);
        k_gjk_class_start<T><<<1, 32, 0, st_>>>(d);
        k_gjk_class_scatter<T><<<gp, 256, 0, st_>>>(d, pv);
        PK_CUDA(mark(kStages + 2));
        k_narrow_gjk<T><<<grid(cfg_.pair_cap) * tune_.narrow_grid, 128, 0, st_>>>(d, pv);
        PK_CUDA(mark(kStages + 3));
        k_narrow_epa<T><<<grid(cfg_.pair_cap) * tune_.narrow_grid, 128, 0, st_>>>(d, pv);
        PK_CUDA(mark(6));
        k_contact_setup<T><<<gp, 256, 0, st_>>>(d, pk, pv, dt);
        if (joint_cap_ > 0) k_joint_setup<T><<<grid(joint_cap_), 128, 0, st_>>>(d, dt);
        PK_CUDA(mark(7));
        for (int gw : grid_worlds_)
        {
            // one cooperative launch per world too large for a CTA
            int wid = gw;
            GridScratch *gs = grid_scratch_;
            void *args[] = {&d, const_cast<uint64_t **>(&pv), &wid, &gs};
            PK_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<void *>(k_solve_grid<T>), dim3(grid_blocks_), dim3(256),
                                                args, 0, st_));
        }
        // the large worlds' launch (the solver's critical path) and the smaller worlds' launches run
        // side by side: the small worlds fill the SMs the large ones leave idle. Worlds are disjoint.
        const bool side = big_worlds_ > 0 && cfg_.max_worlds > big_worlds_;
        cudaStream_t sst = side ? st2_ : st_;
        if (side)
        {
            PK_CUDA(cudaEventRecord(fork_, st_));
            PK_CUDA(cudaStreamWaitEvent(st2_, fork_, 0));
        }
        if (big_worlds_ > 0)
            launch_solve(big_worlds_, tune_.big_threads > 0 ? tune_.big_threads : tune_.solve_threads, big_smem_, d, pv,
                         0, big_cache_, st_);
        if (ngroups() > 0 && joint_cap_ == 0 && tune_.group_warp)
            k_solve_group<T, true><<<ngroups(), tune_.group_threads, sizeof(Vel<T>) * size_t(group_cache_), sst>>>(
                d, pv, goff_dev_, group_cache_);
        else if (ngroups() > 0 && joint_cap_ == 0)
            k_solve_group<T, false><<<ngroups(), tune_.group_threads, sizeof(Vel<T>) * size_t(group_cache_), sst>>>(
                d, pv, goff_dev_, group_cache_);
        else if (cfg_.max_worlds > big_worlds_)
            launch_solve(cfg_.max_worlds - big_worlds_, tune_.solve_threads,
                         sizeof(Vel<T>) * size_t(tune_.small_world), d, pv, big_worlds_, tune_.small_world, sst);
        if (side)
        {
            PK_CUDA(cudaEventRecord(join_, st2_));
            PK_CUDA(cudaStreamWaitEvent(st_, join_, 0));
        }
        PK_CUDA(mark(8));
        k_integrate_pos<T><<<gb, 256, 0, st_>>>(d, dt);
        k_finish<T><<<gp, 256, 0, st_>>>(d, pk, pv);
        PK_CUDA(mark(9));
        if (timing_ && !capturing_) ++timed_steps_;
        PK_CUDA(cudaGetLastError());
        return 0;
    }
};

} // namespace pk
