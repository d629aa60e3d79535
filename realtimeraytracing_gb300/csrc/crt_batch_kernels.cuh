// Included at the end of crt_build.cu (it reuses that file's PLOC tile,
// layout and grid-barrier device code).
//
// Many scenes in one pipeline (config 2): every stage is one launch over all
// scenes, the PLOC iterations of all scenes run in lockstep inside one
// persistent cooperative kernel, and the whole build + trace can be captured
// into a CUDA graph and replayed.  Each scene's BVH is bit-identical to the
// one crt_build makes for that scene alone (same codes, same sort order,
// same PLOC decisions), because every kernel only sees its scene's data
// through per-scene offsets.
#pragma once

namespace crt {

// Per-scene reduction state of the scene box (all-zero initial state: the
// minimum keys are stored inverted so a memset resets them).
struct BatchBoxState {
    unsigned long long key_max[3];
    unsigned long long key_min_inv[3];
    unsigned int blocks_done;
    unsigned int pad0;
    float cube_min[3];
    float cube_len[3];
    float pad[2];
};

struct Chunk {
    uint32_t scene, begin, end, pad;
};

constexpr uint32_t kBoxChunk = 256 * 16;

__device__ __forceinline__ uint32_t scene_of(const uint32_t* off, uint32_t n, uint32_t i) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void tri_extent_b(const TriRec& t, const float* __restrict__ models, float hi[3], float lo[3]) {
    const float* M = models + 16 * (t.model & (kMaxModels - 1));
    const float4 p0 = mat_vec(M, t.p0), p1 = mat_vec(M, t.p1), p2 = mat_vec(M, t.p2);
    hi[0] = max_std(p0.x, max_std(p1.x, p2.x));
    hi[1] = max_std(p0.y, max_std(p1.y, p2.y));
    hi[2] = max_std(p0.z, max_std(p1.z, p2.z));
    lo[0] = min_std(p0.x, min_std(p1.x, p2.x));
    lo[1] = min_std(p0.y, min_std(p1.y, p2.y));
    lo[2] = min_std(p0.z, min_std(p1.z, p2.z));
}

// Scene boxes (bvh.cpp:235-251 per scene, leftmost arg-max as in the single
// scene kernel), then the cube (bvh.cpp:253-303) by each scene's last chunk.
__global__ void __launch_bounds__(256) batch_box_kernel(const crt_triangle* __restrict__ tris, const Chunk* __restrict__ chunks,
                                                        const float* __restrict__ models, BatchBoxState* states,
                                                        BatchScene* scenes, uint32_t* err) {
    const Chunk ch = chunks[blockIdx.x];
    BatchBoxState* st = states + ch.scene;
    unsigned long long kmax[3] = {0ull, 0ull, 0ull}, kmin[3] = {0ull, 0ull, 0ull};  // kmin inverted
    bool bad = false;
    for (uint32_t i = ch.begin + threadIdx.x; i < ch.end; i += 256) {
        const TriRec t = load_tri(tris, i);
        bad |= t.model >= kMaxModels;
        float hi[3], lo[3];
        tri_extent_b(t, models, hi, lo);
        const uint32_t li = i - scenes[ch.scene].tri_off;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (hi[a] == hi[a]) {
                const unsigned long long k = (static_cast<unsigned long long>(ordered_key(hi[a])) << 32) | (0xFFFFFFFFu - li);
                kmax[a] = k > kmax[a] ? k : kmax[a];
            }
            if (lo[a] == lo[a]) {
                const unsigned long long k = ~((static_cast<unsigned long long>(ordered_key(lo[a])) << 32) | li);
                kmin[a] = k > kmin[a] ? k : kmin[a];
            }
        }
    }
    if (bad) raise_error(err, kDevBadModel);
#pragma unroll
    for (int a = 0; a < 3; ++a)
        for (int m = 16; m > 0; m >>= 1) {
            const unsigned long long x = __shfl_xor_sync(0xFFFFFFFFu, kmax[a], m), y = __shfl_xor_sync(0xFFFFFFFFu, kmin[a], m);
            kmax[a] = x > kmax[a] ? x : kmax[a];
            kmin[a] = y > kmin[a] ? y : kmin[a];
        }
    __shared__ unsigned long long s_k[6][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) { s_k[a][warp] = kmax[a]; s_k[3 + a][warp] = kmin[a]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int a = threadIdx.x;
        unsigned long long v = s_k[a][0];
        for (int w = 1; w < 8; ++w) v = s_k[a][w] > v ? s_k[a][w] : v;
        if (a < 3) atomicMax(&st->key_max[a], v); else atomicMax(&st->key_min_inv[a - 3], v);
    }
    __shared__ bool s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(&st->blocks_done, 1u) == scenes[ch.scene].n_chunks - 1);
    __syncthreads();
    if (!s_last || threadIdx.x != 0) return;
    __threadfence();
    const uint32_t base = scenes[ch.scene].tri_off;
    const float kInf = __int_as_float(0x7F800000);
    float smin[3], smax[3];
    for (int a = 0; a < 3; ++a) {
        const unsigned long long kx = atomicAdd(&st->key_max[a], 0ull);
        const unsigned long long kn = ~atomicAdd(&st->key_min_inv[a], 0ull);
        smax[a] = -kInf;
        smin[a] = kInf;
        float hi[3], lo[3];
        if (kx != 0ull) {
            tri_extent_b(load_tri(tris, base + (0xFFFFFFFFu - static_cast<uint32_t>(kx))), models, hi, lo);
            smax[a] = hi[a];
        }
        if (kn != ~0ull) {
            tri_extent_b(load_tri(tris, base + static_cast<uint32_t>(kn)), models, hi, lo);
            smin[a] = lo[a];
        }
    }
    float cmn[3] = {smin[0], smin[1], smin[2]}, cmx[3] = {smax[0], smax[1], smax[2]};
    const float dX = smax[0] - smin[0], dY = smax[1] - smin[1], dZ = smax[2] - smin[2];
    float maxDist = 0.f;
    int axis;
    if (dX > maxDist) { maxDist = dX; axis = 0; }
    else if (dY > maxDist) { maxDist = dY; axis = 1; }
    else { maxDist = dZ; axis = 2; }
    const float dist[3] = {dX, dY, dZ};
    for (int a = 0; a < 3; ++a) {
        if (a == axis) continue;
        const float delta = (maxDist - dist[a]) / 2.f;
        cmx[a] += delta;
        cmn[a] -= delta;
    }
    for (int a = 0; a < 3; ++a) {
        st->cube_min[a] = cmn[a];
        st->cube_len[a] = cmx[a] - cmn[a];
    }
    scenes[ch.scene].abs_eps = scene_abs_eps(smin, smax);
}

__device__ __forceinline__ uint32_t expand_bits_b(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__device__ __forceinline__ uint32_t to_u10_b(float x) {
    x = min_std(max_std(x * 1024.0f, 0.0f), 1023.0f);
    return __float2uint_rz(x);
}

template <int BITS>
__global__ void __launch_bounds__(256) batch_morton_kernel(const crt_triangle* __restrict__ tris, const Chunk* __restrict__ chunks,
                                                           const float* __restrict__ models_third,
                                                           const BatchBoxState* __restrict__ states,
                                                           uint32_t* __restrict__ codes, uint32_t* __restrict__ hist) {
    constexpr int RADIX = 1 << BITS;
    constexpr int PASSES = (30 + BITS - 1) / BITS;
    __shared__ uint32_t s_hist[PASSES * RADIX];
    for (int i = threadIdx.x; i < PASSES * RADIX; i += blockDim.x) s_hist[i] = 0u;
    __syncthreads();
    const Chunk ch = chunks[blockIdx.x];
    const BatchBoxState* st = states + ch.scene;
    const float cmx = st->cube_min[0], cmy = st->cube_min[1], cmz = st->cube_min[2];
    const float lx = st->cube_len[0], ly = st->cube_len[1], lz = st->cube_len[2];
    for (uint32_t i = ch.begin + threadIdx.x; i < ch.end; i += 256) {
        const TriRec t = load_tri(tris, i);
        const float* M3 = models_third + 16 * (t.model & (kMaxModels - 1));
        float4 s;
        s.x = t.p0.x + t.p1.x + t.p2.x;
        s.y = t.p0.y + t.p1.y + t.p2.y;
        s.z = t.p0.z + t.p1.z + t.p2.z;
        s.w = t.p0.w + t.p1.w + t.p2.w;
        const float4 c = mat_vec(M3, s);
        const float nx = (c.x - cmx) / lx, ny = (c.y - cmy) / ly, nz = (c.z - cmz) / lz;
        const uint32_t code = (expand_bits_b(to_u10_b(nx)) << 2) | (expand_bits_b(to_u10_b(ny)) << 1) | expand_bits_b(to_u10_b(nz));
        codes[i] = code;
#pragma unroll
        for (int p = 0; p < PASSES; ++p) atomicAdd(&s_hist[p * RADIX + ((code >> (p * BITS)) & (RADIX - 1))], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < PASSES * RADIX; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

// Leaf clusters per scene (as leaf_init_kernel), plus each scene's first
// PLOC record and, for one-triangle scenes, their single output node.
__global__ void __launch_bounds__(256) batch_leaf_init_kernel(const crt_triangle* __restrict__ tris, uint32_t n_total,
                                                              BatchScene* scenes, uint32_t n_scenes,
                                                              const float* __restrict__ models,
                                                              const uint32_t* __restrict__ perm_global,
                                                              uint32_t* __restrict__ perm_local, float4* __restrict__ node_box,
                                                              float4* __restrict__ clusters,
                                                              float4* __restrict__ xtri_sorted, float4* __restrict__ xtri,
                                                              uint32_t* __restrict__ leaf_of_tri, uint2* __restrict__ it,
                                                              crt_bvh_node* __restrict__ nodes, uint32_t* err) {
    __shared__ uint32_t s_off[kMaxBatchScenes];
    for (uint32_t k = threadIdx.x; k < n_scenes; k += 256) s_off[k] = scenes[k].tri_off;
    __syncthreads();
    const uint32_t i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n_total) return;
    const uint32_t s = scene_of(s_off, n_scenes, i);
    const BatchScene sc = scenes[s];
    const uint32_t li = i - sc.tri_off;
    const uint32_t tg = perm_global[i];
    const uint32_t tl = tg - sc.tri_off;
    if (tg < sc.tri_off || tl >= sc.n_tris) { raise_corrupt(err, 6, i, tg); return; }
    if (li == 0) {
        it[sc.it_off] = make_uint2(sc.n_tris, sc.n_tris);
        scenes[s].iters = sc.n_tris > 1 ? 0u : 1u;   // one-triangle scenes need no iteration
    }
    perm_local[i] = tl;
    const TriRec t = load_tri(tris, tg);
    const float* M = models + 16 * (t.model & (kMaxModels - 1));
    const float4 p0 = mat_vec(M, t.p0), p1 = mat_vec(M, t.p1), p2 = mat_vec(M, t.p2);
    float4 mn, mx;
    mn.x = min_std(p0.x, min_std(p1.x, p2.x));
    mn.y = min_std(p0.y, min_std(p1.y, p2.y));
    mn.z = min_std(p0.z, min_std(p1.z, p2.z));
    mx.x = max_std(p0.x, max_std(p1.x, p2.x));
    mx.y = max_std(p0.y, max_std(p1.y, p2.y));
    mx.z = max_std(p0.z, max_std(p1.z, p2.z));
    const size_t nb = 2 * (static_cast<size_t>(sc.node_off) + li);
    node_box[nb] = make_float4(mn.x, mn.y, mn.z, __uint_as_float(tl));
    node_box[nb + 1] = make_float4(mx.x, mx.y, mx.z, 0.f);
    clusters[2 * static_cast<size_t>(i)] = make_float4(mn.x, mn.y, mn.z, __uint_as_float(li));
    clusters[2 * static_cast<size_t>(i) + 1] = make_float4(mx.x, mx.y, mx.z, __uint_as_float(1u));
    // sorted order; the layout moves them into tree order (a one-triangle
    // scene's single leaf is in both orders at once)
    float4* xo = (sc.n_tris == 1 ? xtri : xtri_sorted) + 3 * static_cast<size_t>(i);
    xo[0] = make_float4(p0.x, p0.y, p0.z, __uint_as_float(tl));
    xo[1] = make_float4(p1.x, p1.y, p1.z, __uint_as_float(t.model));
    xo[2] = make_float4(p2.x, p2.y, p2.z, 0.f);
    if (sc.n_tris == 1) {
        leaf_of_tri[sc.tri_off] = 0u;
        float4* o = reinterpret_cast<float4*>(nodes + sc.node_off);
        o[0] = make_float4(mn.x, mn.y, mn.z, 0.f);
        o[1] = make_float4(mx.x, mx.y, mx.z, 0.f);
        reinterpret_cast<uint4*>(o)[2] = make_uint4(tl, 0u, 0u, 0u);
    }
}

// PLOC for all scenes in lockstep, then every scene's DFS layout.  Each
// iteration: every block derives the running scenes' tile counts (a scene
// converged once its iteration count is set), takes tiles from one ticket
// counter, maps a ticket to (scene, tile) and runs the single-scene tile
// code on that scene's slices.  A grid barrier separates iterations.
template <int TILE, int BLOCK, int MAXR>
__global__ void __launch_bounds__(BLOCK, kPlocBlocksPerSm) batch_ploc_kernel(BatchScene* scenes, uint32_t n_scenes, float4* ca, float4* cb,
                                                           float4* node_box, uint4* node_kids, uint2* it, int R,
                                                           unsigned long long* lookback, uint32_t lb_cap, uint32_t* tickets,
                                                           uint2* pf, crt_bvh_node* nodes, float4* wide, float4* wide_wt,
                                                           uint8_t* depth_odd, LeafOut lv, unsigned long long* bar,
                                                           uint32_t max_iters, uint32_t* err, uint32_t spin_limit) {
    __shared__ PlocSmem<TILE, BLOCK, MAXR> S;
    unsigned long long bar_target = 0;  // grid barriers passed x gridDim (thread 0)
    __shared__ uint32_t s_tile_pre[kMaxBatchScenes + 1];
    __shared__ uint32_t s_n[kMaxBatchScenes];
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_running;
    int iter = 0;
    for (;; ++iter) {
        __syncthreads();
        if (threadIdx.x == 0) s_running = 0;
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < n_scenes; k += BLOCK) {
            const uint32_t done = __ldcg(&scenes[k].iters);
            uint32_t n = 1;
            if (done == 0u) {
                n = __ldcg(it + scenes[k].it_off + iter).x;
                if (n > 1) atomicAdd(&s_running, 1u);
            }
            s_n[k] = n;
        }
        __syncthreads();
        if (s_running == 0) break;
        if (static_cast<uint32_t>(iter) >= max_iters) { raise_error(err, kDevIterLimit); return; }
        // Once every running scene fits in one tile, each block finishes whole
        // scenes alone (their remaining iterations, one tile each, with block
        // barriers only) and one grid barrier ends the PLOC phase.
        if (threadIdx.x == 0) {
            uint32_t big = 0;
            for (uint32_t k = 0; k < n_scenes; ++k) big += s_n[k] > ploc_own(R) ? 1u : 0u;
            s_tile = big;
        }
        __syncthreads();
        if (s_tile == 0u) {
            for (uint32_t sc = blockIdx.x; sc < n_scenes; sc += gridDim.x) {
                if (s_n[sc] <= 1u) continue;  // finished before this iteration
                const BatchScene B = scenes[sc];
                // the scene's remaining iterations on shared memory (ploc_tail);
                // its iteration count cannot exceed the scene's N - 1
                const float4* cin = ((iter & 1) ? cb : ca) + 2 * static_cast<size_t>(B.tri_off);
                const int k = ploc_tail<TILE, BLOCK, MAXR>(S, iter, cin, node_box + 2 * static_cast<size_t>(B.node_off),
                                                          node_kids + B.tri_off, it + B.it_off, B.n_tris, R, err);
                if (threadIdx.x == 0) scenes[sc].iters = static_cast<uint32_t>(k);
                __syncthreads();
            }
            if (!grid_barrier(bar, bar_target, err, spin_limit)) return;
            break;
        }
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (uint32_t k = 0; k < n_scenes; ++k) {
                s_tile_pre[k] = run;
                run += s_n[k] > 1 ? (s_n[k] + ploc_own(R) - 1) / ploc_own(R) : 0u;
            }
            s_tile_pre[n_scenes] = run;
        }
        __syncthreads();
        const uint32_t total = s_tile_pre[n_scenes];
        for (;;) {
            __syncthreads();
            if (threadIdx.x == 0) s_tile = atomicAdd(&tickets[iter & 1], 1u);
            __syncthreads();
            const uint32_t g = s_tile;
            if (g >= total) break;
            if (g == 0 && threadIdx.x == 0) tickets[(iter + 1) & 1] = 0u;
            uint32_t lo = 0, hi = n_scenes - 1;  // scene whose tile range holds g
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (s_tile_pre[mid] <= g) lo = mid; else hi = mid - 1;
            }
            const uint32_t sc = lo, tile = g - s_tile_pre[sc];
            const BatchScene B = scenes[sc];
            const uint2 cur = make_uint2(s_n[sc], __ldcg(it + B.it_off + iter).y);
            float4* cin = ((iter & 1) ? cb : ca) + 2 * static_cast<size_t>(B.tri_off);
            float4* cout = ((iter & 1) ? ca : cb) + 2 * static_cast<size_t>(B.tri_off);
            unsigned long long* lb_cur = lookback + static_cast<size_t>(iter & 1) * lb_cap + B.lb_off;
            unsigned long long* lb_next = lookback + static_cast<size_t>((iter + 1) & 1) * lb_cap + B.lb_off;
            ploc_tile<TILE, BLOCK, MAXR>(S, tile, cur, iter, cin, cout, node_box + 2 * static_cast<size_t>(B.node_off),
                                         node_kids + B.tri_off, it + B.it_off, B.n_tris, R, lb_cur, lb_next, err, spin_limit);
            if ((tile + 1) * ploc_own(R) >= cur.x && threadIdx.x == 0) {  // the scene's last tile wrote its next record
                if (it[B.it_off + iter + 1].x <= 1u) scenes[sc].iters = static_cast<uint32_t>(iter + 1);
            }
        }
        if (!grid_barrier(bar, bar_target, err, spin_limit)) return;
    }
    // DFS layout: step r handles level (iters - 1 - r) of every scene that has
    // it, recording node ids by DFS position in dfs (the first cluster buffer,
    // free now); then every position is emitted in order.
    uint32_t* dfs = reinterpret_cast<uint32_t*>(ca);
    uint32_t max_it = 0;
    for (uint32_t k = 0; k < n_scenes; ++k) max_it = max(max_it, __ldcg(&scenes[k].iters));
    for (uint32_t r = 0; r < max_it; ++r) {
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (uint32_t k = 0; k < n_scenes; ++k) {
                s_tile_pre[k] = run;
                const uint32_t K = __ldcg(&scenes[k].iters);
                if (scenes[k].n_tris > 1 && K > r) {
                    const uint32_t lv = K - 1 - r;
                    const uint32_t o = scenes[k].it_off;
                    run += __ldcg(it + o + lv + 1).y - __ldcg(it + o + lv).y;
                }
            }
            s_tile_pre[n_scenes] = run;
        }
        __syncthreads();
        const uint32_t total = s_tile_pre[n_scenes];
        for (uint32_t q = blockIdx.x * BLOCK + threadIdx.x; q < total; q += gridDim.x * BLOCK) {
            uint32_t lo = 0, hi = n_scenes - 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (s_tile_pre[mid] <= q) lo = mid; else hi = mid - 1;
            }
            const BatchScene B = scenes[lo];
            const uint32_t lv = B.iters - 1 - r;
            const uint32_t X = __ldcg(it + B.it_off + lv).y + (q - s_tile_pre[lo]);
            layout_down(X, node_kids + B.tri_off, pf + B.tri_off, B.n_tris,
                        dfs + B.node_off, err);
        }
        if (!grid_barrier(bar, bar_target, err, spin_limit)) return;
    }
    // every DFS position of every scene with more than one triangle, in order
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t k = 0; k < n_scenes; ++k) {
            s_tile_pre[k] = run;
            if (scenes[k].n_tris > 1) run += 2 * scenes[k].n_tris - 1;
        }
        s_tile_pre[n_scenes] = run;
    }
    __syncthreads();
    const uint32_t total_slots = s_tile_pre[n_scenes];
    for (uint32_t q = blockIdx.x * BLOCK + threadIdx.x; q < total_slots; q += gridDim.x * BLOCK) {
        uint32_t lo = 0, hi = n_scenes - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (s_tile_pre[mid] <= q) lo = mid; else hi = mid - 1;
        }
        const BatchScene B = scenes[lo];
        const LeafOut slv{lv.xtri_sorted + 3 * static_cast<size_t>(B.tri_off), lv.xtri + 3 * static_cast<size_t>(B.tri_off),
                          lv.leaf_of_tri + B.tri_off};
        layout_emit(q - s_tile_pre[lo], node_box + 2 * static_cast<size_t>(B.node_off), node_kids + B.tri_off,
                    pf + B.tri_off, B.n_tris, dfs + B.node_off, nodes + B.node_off,
                    wide + 4 * static_cast<size_t>(B.wide_off), wide_wt + 4 * static_cast<size_t>(B.wide_off),
                    depth_odd + B.wide_off, slv, B.abs_eps, err);
    }
}

// ------------------------------------------------------------------ launchers
int batch_ploc_grid() {
    static int grid = -1;
    if (grid < 0) {
        int per_sm = 0, dev = 0, sms = kNumSms, coop = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                        &per_sm, batch_ploc_kernel<kPlocSpan, 256, kPlocMaxRadius>, 256, 0) == cudaSuccess && per_sm > 0)
            grid = (per_sm < kPlocBlocksPerSm ? per_sm : kPlocBlocksPerSm) * sms;
        else
            grid = 0;
        cudaGetLastError();
    }
    return grid;
}

void launch_batch_box(const crt_triangle* tris, const void* chunks, uint32_t n_chunks, const float* models, void* states,
                      BatchScene* scenes, uint32_t* err, cudaStream_t s) {
    batch_box_kernel<<<n_chunks, 256, 0, s>>>(tris, static_cast<const Chunk*>(chunks), models,
                                              static_cast<BatchBoxState*>(states), scenes, err);
}

void launch_batch_morton(const crt_triangle* tris, const void* chunks, uint32_t n_chunks, const float* models_third,
                         const void* states, uint32_t* codes, uint32_t* hist, int bits, cudaStream_t s) {
    if (bits == 4)
        batch_morton_kernel<4><<<n_chunks, 256, 0, s>>>(tris, static_cast<const Chunk*>(chunks), models_third,
                                                        static_cast<const BatchBoxState*>(states), codes, hist);
    else
        batch_morton_kernel<8><<<n_chunks, 256, 0, s>>>(tris, static_cast<const Chunk*>(chunks), models_third,
                                                        static_cast<const BatchBoxState*>(states), codes, hist);
}

void launch_batch_leaf_init(const crt_triangle* tris, uint32_t n_total, BatchScene* scenes, uint32_t n_scenes,
                            const float* models, const uint32_t* perm_global, uint32_t* perm_local, float4* node_box,
                            float4* clusters, float4* xtri_sorted, float4* xtri, uint32_t* leaf_of_tri, uint2* it,
                            crt_bvh_node* nodes,
                            uint32_t* err, cudaStream_t s) {
    batch_leaf_init_kernel<<<(n_total + 255) / 256, 256, 0, s>>>(tris, n_total, scenes, n_scenes, models, perm_global,
                                                                 perm_local, node_box, clusters, xtri_sorted, xtri,
                                                                 leaf_of_tri, it, nodes,
                                                                 err);
}

cudaError_t launch_batch_ploc(BatchScene* scenes, uint32_t n_scenes, float4* ca, float4* cb, float4* node_box,
                              uint4* node_kids, uint2* it, int radius, unsigned long long* lookback, uint32_t lb_cap,
                              uint32_t* tickets, uint2* pf, crt_bvh_node* nodes, float4* wide, float4* wide_wt,
                              uint8_t* depth_odd, LeafOut lv, unsigned long long* bar, uint32_t max_iters, uint32_t* err,
                              uint32_t spin_limit, cudaStream_t s) {
    const int grid = batch_ploc_grid();
    if (grid <= 0) return cudaErrorNotSupported;
    void* args[] = {&scenes, &n_scenes, &ca, &cb, &node_box, &node_kids, &it, &radius, &lookback, &lb_cap, &tickets,
                    &pf, &nodes, &wide, &wide_wt, &depth_odd, &lv, &bar, &max_iters, &err, &spin_limit};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(batch_ploc_kernel<kPlocSpan, 256, kPlocMaxRadius>),
                                       dim3(grid), dim3(256), args, 0, s);
}

size_t batch_box_state_bytes() { return sizeof(BatchBoxState); }
size_t batch_chunk_bytes() { return sizeof(Chunk); }
uint32_t batch_box_chunk() { return kBoxChunk; }

}  // namespace crt
