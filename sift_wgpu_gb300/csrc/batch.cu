// batch.cu — the batched form: one run over many images of any sizes.
//
// The (image, octave) pairs of a batch are entries of one table, image-major
// (entry = image * num_octaves + octave), laid out back to back in one u8
// level arena (the batch keeps every level only as its u8 plane). Each stage
// of the hot path is one launch over the flattened work of all images:
//
//   pyramid      one launch per (octave, level), over the tiles (or rows) of
//                that octave of every image; each octave's levels above S run
//                on a second stream beside the next octave
//   extrema      one launch over the tiles of every entry
//   candidates   one prefix scan over every entry's mask words: the mask
//                words are image-major too, so the candidates come out in
//                (image, octave, layer, y, x) order, each image's in the
//                reference order
//   refinement, orientation, oriented keypoints, descriptors: one launch
//                each over the batch's single lists
//   export       each image's range of the output and the octave fields
//
// The whole run is captured as one CUDA graph per batch geometry and replayed;
// the images are copied in before the replay, and the run writes its results
// (descriptors from the descriptor stage, keypoints and per-image ranges from
// the export) into mapped host memory. Results are the single-image
// engine's, bit for bit: the same tile bodies and per-item arithmetic run on
// the same values.
#include "engine.h"

namespace sift {

int blur_level_tiles(int W, int H);
int blur_col_tiles(int W, int H);
int lanczos_tiles(int nW, int nH);
size_t batch_lz_bytes();
void batch_lz_fill(void* out, int vtab, int vw, int htab, int hw, const LanczosUniform& uni);
int launch_blur_level_flat(const BatchPyr& bp, uint8_t* tmp, int o, int s, int r, int n_img,
                           const uint32_t* fused_pref, uint32_t n_fused, const uint32_t* rows_pref, uint32_t n_rows,
                           int max_w, const uint32_t* cols_pref, uint32_t n_cols, const float* wts,
                           const float* lut255, cudaStream_t st, int* launches, int fused_max_radius);
int launch_lanczos_flat(const BatchPyr& bp, int o, int n_img, const uint32_t* pref, uint32_t n_tiles,
                        const void* lz, const int* itab, const float* ftab, cudaStream_t st);

namespace {

// Each image's first output keypoint (ranges[i], ranges[n_img] = total) and
// the octave field of every output keypoint (its entry's octave), written to
// the mapped host buffer too: counters, ranges and the first cap_x keypoints
// (the descriptor stage writes the first cap_x descriptors there itself).
__global__ void k_batch_export(const OctaveDev* __restrict__ ents, int O, int n_img, long long total_words,
                               const uint32_t* __restrict__ cand_off, const uint32_t* __restrict__ ori_off,
                               const Counters* __restrict__ ctr, uint32_t cap_cand, Keypoint* __restrict__ oriented,
                               uint32_t cap_ori, Counters* hctr, uint32_t* hranges, Keypoint* hkps, uint32_t cap_x) {
    chain_wait();
    const OctCounters& oc = ctr->oct[0];
    const uint32_t n_cand = min(oc.n_cand, cap_cand), n_ori = min(oc.n_ori, cap_ori);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    constexpr uint32_t kCtrWords = sizeof(Counters) / 4;
    if (tid < kCtrWords) reinterpret_cast<uint32_t*>(hctr)[tid] = reinterpret_cast<const uint32_t*>(ctr)[tid];
    if (tid <= (uint32_t)n_img) {
        const long long w = tid < (uint32_t)n_img ? ents[tid * O].word_base : total_words;
        const uint32_t c = w < total_words ? min(cand_off[w], n_cand) : n_cand;
        hranges[tid] = c < n_cand ? min(ori_off[c], n_ori) : n_ori;
    }
    for (uint32_t j = tid; j < n_ori; j += stride) {
        Keypoint k = oriented[j];
        k.octave = ents[k.octave].octave;
        oriented[j] = k;
        if (j < cap_x) hkps[j] = k;
    }
}

}  // namespace

struct BatchEngine {
    SiftCudaParams p{};
    SiftCudaOptions opt{};
    cudaStream_t st = nullptr, st2 = nullptr;
    std::vector<cudaEvent_t> ev_lvl;
    cudaEvent_t ev_side = nullptr;

    // geometry of the current batch
    std::vector<std::pair<uint32_t, uint32_t>> dims;
    int N = 0, O = 0, S = 0;
    std::vector<OctaveDev> ents;
    std::vector<long long> img_off;
    std::vector<int> img_pitch;
    long long total_words = 0;
    int max_w = 0;
    struct OctPref {
        size_t fused, rows, cols, lz;  // offsets (u32 elements) in d_pref
        uint32_t n_fused, n_rows, n_cols, n_lz;
    };
    std::vector<OctPref> opref;
    size_t ex_pref = 0;
    uint32_t n_ex = 0;
    LevelBlur base{};
    std::vector<std::vector<LevelBlur>> lv;
    size_t lut_off = 0;

    DevMem d_img, d_U, d_tmp, d_tmp2, d_ents, d_pref, d_imgaddr, d_imgpitch, d_wts, d_ltab, d_lw, d_lz;
    // the device reads pageable host memory coherently (Grace's address
    // translation): the base level then reads the caller's images in place
    bool host_reads = false;
    std::vector<unsigned long long> h_addr;
    std::vector<int> h_pitch;
    DevMem d_words, d_cand_off, d_scan, d_cands, d_refined, d_keep, d_ori_angle, d_ori_count, d_ori_off, d_oriented,
        d_desc, d_ctr;
    HostPinned h_ctr;
    // Mapped host buffer the run writes its results into: Counters | ranges
    // (n + 1) | keypoints[cap_x] | descriptors[cap_x]; sized from the last
    // count, grown (with a re-run) when a batch has more keypoints.
    HostPinned hx;
    uint32_t cap_x = 0;
    Counters* hx_dctr = nullptr;
    uint32_t* hx_dranges = nullptr;
    Keypoint* hx_dkps = nullptr;
    float* hx_ddesc = nullptr;
    size_t hx_ranges_off() const { return align_up(sizeof(Counters), 256); }
    size_t hx_kps_off() const { return hx_ranges_off() + align_up(sizeof(uint32_t) * (size_t)(N + 1), 256); }
    size_t hx_desc_off() const { return hx_kps_off() + align_up(sizeof(Keypoint) * (size_t)cap_x, 256); }
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
    float device_ms = 0.0f;
    uint32_t cap_cand = 0, cap_ori = 0;
    size_t scan_words = 0, scan_b = 0;  // scan state: words scan at 0, orientation-count scan at scan_b
    uint32_t n_out = 0;
    bool images_in_place = false;  // the last run read the caller's images in place

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    uint32_t launches = 0, graph_launches = 0;

    ~BatchEngine() {
        drop_graph();
        for (auto e : ev_lvl)
            if (e) cudaEventDestroy(e);
        if (ev_side) cudaEventDestroy(ev_side);
        if (ev_t0) cudaEventDestroy(ev_t0);
        if (ev_t1) cudaEventDestroy(ev_t1);
        if (st2) cudaStreamDestroy(st2);
        if (st) cudaStreamDestroy(st);
    }
    void drop_graph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        gexec = nullptr;
        graph = nullptr;
    }
    EntryTable tab() const { return EntryTable{d_ents.as<OctaveDev>(), N * O, S}; }
    BatchPyr bpyr() const {
        return BatchPyr{d_U.as<uint8_t>(), d_ents.as<OctaveDev>(), O, S, d_imgaddr.as<unsigned long long>(),
                        d_imgpitch.as<int>()};
    }
    const uint32_t* pref(size_t off) const { return d_pref.as<uint32_t>() + off; }

    int init() {
        CK(cudaSetDevice(opt.device), "cudaSetDevice");
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
        CK(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking), "cudaStreamCreate");
        ev_lvl.assign(kMaxOctaves, nullptr);
        for (auto& e : ev_lvl) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaEventCreateWithFlags(&ev_side, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaEventCreate(&ev_t0), "cudaEventCreate");
        CK(cudaEventCreate(&ev_t1), "cudaEventCreate");
        CK(d_ctr.ensure(sizeof(Counters)), "cudaMalloc(counters)");
        CK(h_ctr.ensure(sizeof(Counters)), "cudaHostAlloc(counters)");
        int pageable = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, opt.device) != cudaSuccess) pageable = 0;
        host_reads = pageable == 1;
        return 0;
    }

    // Arenas, tables and work-list prefixes for images of these sizes.
    int ensure_geometry(const std::vector<std::pair<uint32_t, uint32_t>>& d) {
        if (!ents.empty() && d == dims) return 0;
        drop_graph();
        O = (int)p.num_octaves;
        S = (int)p.num_intervals;
        if (O > kMaxOctaves) return fail(SIFT_CUDA_ERR_UNSUPPORTED, "num_octaves above 16 is not supported");
        N = (int)d.size();
        ents.assign((size_t)N * O, OctaveDev{});
        img_off.assign(N, 0);
        img_pitch.assign(N, 0);
        size_t uoff = 0, toff = 0, ioff = 0;
        long long wbase = 0;
        max_w = 0;
        for (int i = 0; i < N; ++i) {
            img_pitch[i] = (int)align_up(std::max<uint32_t>(d[i].first, 1), 128);
            img_off[i] = (long long)ioff;
            ioff += (size_t)img_pitch[i] * std::max<uint32_t>(d[i].second, 1);
            uint32_t ow = d[i].first, oh = d[i].second;
            for (int o = 0; o < O; ++o) {
                OctaveDev& od = ents[(size_t)i * O + o];
                od.W = (int)ow;
                od.H = (int)oh;
                od.pitch = (int)align_up(std::max<uint32_t>(ow, 1), 32);
                od.nw = (int)((ow + 31) / 32);
                od.plane = (long long)od.pitch * oh;
                od.u_off = od.g_off = (long long)uoff;
                od.t_off = (long long)toff;
                od.word_base = wbase;
                od.octave = o;
                od.image = i;
                uoff += (size_t)od.plane * (S + 3);
                toff += align_up((size_t)od.plane, 256);
                wbase += (long long)S * oh * od.nw;
                max_w = std::max(max_w, (int)ow);
                ow /= 2;
                oh /= 2;
            }
        }
        total_words = wbase;
        // blur weights (the same for every image), v / 255 table
        BlurPlan bp = blur_plan(p);
        std::vector<float> wts;
        auto add_blur = [&](float sigma) {
            LevelBlur b{sigma, 0, wts.size()};
            if (sigma > 0.0f) {
                auto k = gaussian_kernel(sigma);
                b.radius = (int)(k.size() / 2);
                wts.insert(wts.end(), k.begin(), k.end());
                while (wts.size() % 4) wts.push_back(0.0f);
            }
            return b;
        };
        base = add_blur(bp.base);
        lv.assign(O, {});
        for (int o = 0; o < O; ++o)
            for (int s = 1; s < S + 3; ++s) lv[o].push_back(add_blur(bp.level[o][s - 1]));
        lut_off = wts.size();
        for (int v = 0; v < 256; ++v) wts.push_back((float)v / 255.0f);
        // Lanczos tables per (image, octave) resize
        std::vector<int> itab;
        std::vector<float> ftab;
        std::vector<uint8_t> lz(batch_lz_bytes() * (size_t)std::max(N * O, 1), 0);
        auto max_span = [](const AxisTaps& t) {
            const int T = lanczos_fused_tile(), n = (int)t.left.size();
            int m = 0;
            for (int a = 0; a < n; a += T) {
                const int b = std::min(a + T, n) - 1;
                m = std::max(m, t.left[b] + t.count[b] - t.left[a]);
            }
            return m;
        };
        for (int i = 0; i < N; ++i)
            for (int o = 0; o + 1 < O; ++o) {
                const OctaveDev& a = ents[(size_t)i * O + o];
                const OctaveDev& b = ents[(size_t)i * O + o + 1];
                if (a.W == 0 || a.H == 0 || b.W == 0 || b.H == 0) continue;
                AxisTaps tv = lanczos_axis((uint32_t)a.H, (uint32_t)b.H);
                AxisTaps th = lanczos_axis((uint32_t)a.W, (uint32_t)b.W);
                if (max_span(tv) > lanczos_fused_span() || max_span(th) > lanczos_fused_span())
                    return fail(SIFT_CUDA_ERR_UNSUPPORTED, "a batch image's resize window exceeds the fused tile");
                const int vt = (int)itab.size();
                itab.insert(itab.end(), tv.left.begin(), tv.left.end());
                itab.insert(itab.end(), tv.count.begin(), tv.count.end());
                itab.insert(itab.end(), tv.woff.begin(), tv.woff.end());
                const int vwo = (int)ftab.size();
                ftab.insert(ftab.end(), tv.w.begin(), tv.w.end());
                const int ht = (int)itab.size();
                itab.insert(itab.end(), th.left.begin(), th.left.end());
                itab.insert(itab.end(), th.count.begin(), th.count.end());
                itab.insert(itab.end(), th.woff.begin(), th.woff.end());
                const int hwo = (int)ftab.size();
                ftab.insert(ftab.end(), th.w.begin(), th.w.end());
                LanczosUniform uni{};
                Engine::uniform_2x(th, (uint32_t)a.W, &uni.x0, &uni.x1, uni.wh);
                Engine::uniform_2x(tv, (uint32_t)a.H, &uni.y0, &uni.y1, uni.wv);
                if (uni.x0 >= uni.x1 || uni.y0 >= uni.y1) uni.x0 = uni.x1 = uni.y0 = uni.y1 = 0;
                batch_lz_fill(lz.data() + batch_lz_bytes() * ((size_t)i * O + o), vt, vwo, ht, hwo, uni);
            }
        // work-list prefixes: per octave over the images, and over all entries
        std::vector<uint32_t> pr;
        auto prefix = [&](auto count_of) {
            const size_t off = pr.size();
            uint32_t acc = 0;
            for (int i = 0; i < N; ++i) {
                pr.push_back(acc);
                acc += (uint32_t)count_of(i);
            }
            pr.push_back(acc);
            return std::make_pair(off, acc);
        };
        opref.assign(O, OctPref{});
        for (int o = 0; o < O; ++o) {
            auto at = [&](int i) -> const OctaveDev& { return ents[(size_t)i * O + o]; };
            auto f = prefix([&](int i) { return blur_level_tiles(at(i).W, at(i).H); });
            auto r = prefix([&](int i) { return at(i).W > 0 ? at(i).H : 0; });
            auto c = prefix([&](int i) { return blur_col_tiles(at(i).W, at(i).H); });
            auto z = prefix([&](int i) {
                if (o + 1 >= O || at(i).W == 0 || at(i).H == 0) return 0;
                const OctaveDev& nx = ents[(size_t)i * O + o + 1];
                return lanczos_tiles(nx.W, nx.H);
            });
            opref[o] = OctPref{f.first, r.first, c.first, z.first, f.second, r.second, c.second, z.second};
        }
        ex_pref = pr.size();
        {
            uint32_t acc = 0;
            for (int e = 0; e < N * O; ++e) {
                pr.push_back(acc);
                acc += (uint32_t)extrema_tiles(ents[e].W, ents[e].H);
            }
            pr.push_back(acc);
            n_ex = acc;
        }
        // allocate and upload
        CK(d_img.ensure(std::max<size_t>(ioff, 16)), "cudaMalloc(images)");
        CK(d_U.ensure(uoff + 64), "cudaMalloc(u8 levels)");
        CK(d_tmp.ensure(std::max<size_t>(toff, 16)), "cudaMalloc(tmp)");
        CK(d_tmp2.ensure(std::max<size_t>(toff, 16)), "cudaMalloc(tmp)");
        CK(d_ents.ensure(sizeof(OctaveDev) * std::max<size_t>(ents.size(), 1)), "cudaMalloc(entries)");
        CK(d_pref.ensure(sizeof(uint32_t) * pr.size()), "cudaMalloc(prefixes)");
        CK(d_imgaddr.ensure(sizeof(unsigned long long) * std::max(N, 1)), "cudaMalloc(image table)");
        CK(d_imgpitch.ensure(sizeof(int) * std::max(N, 1)), "cudaMalloc(image table)");
        CK(d_wts.ensure(sizeof(float) * wts.size()), "cudaMalloc(wts)");
        CK(d_ltab.ensure(sizeof(int) * std::max<size_t>(itab.size(), 4)), "cudaMalloc(ltab)");
        CK(d_lw.ensure(sizeof(float) * std::max<size_t>(ftab.size(), 4)), "cudaMalloc(lw)");
        CK(d_lz.ensure(lz.size()), "cudaMalloc(lanczos jobs)");
        const size_t nwb = sizeof(uint32_t) * (size_t)std::max<long long>(total_words, 1);
        CK(d_words.ensure(nwb), "cudaMalloc(words)");
        CK(d_cand_off.ensure(nwb), "cudaMalloc(cand_off)");
        if (!ents.empty())
            CK(cudaMemcpyAsync(d_ents.p, ents.data(), sizeof(OctaveDev) * ents.size(), cudaMemcpyHostToDevice, st),
               "H2D entries");
        CK(cudaMemcpyAsync(d_pref.p, pr.data(), sizeof(uint32_t) * pr.size(), cudaMemcpyHostToDevice, st), "H2D pref");
        CK(cudaMemcpyAsync(d_wts.p, wts.data(), sizeof(float) * wts.size(), cudaMemcpyHostToDevice, st), "H2D wts");
        if (!itab.empty())
            CK(cudaMemcpyAsync(d_ltab.p, itab.data(), sizeof(int) * itab.size(), cudaMemcpyHostToDevice, st), "H2D");
        if (!ftab.empty())
            CK(cudaMemcpyAsync(d_lw.p, ftab.data(), sizeof(float) * ftab.size(), cudaMemcpyHostToDevice, st), "H2D");
        CK(cudaMemcpyAsync(d_lz.p, lz.data(), lz.size(), cudaMemcpyHostToDevice, st), "H2D lanczos jobs");
        CK(cudaStreamSynchronize(st), "table upload");
        dims = d;
        // list capacities: 1/64 of the scanned positions, at least 1024 per entry
        size_t cc = 0;
        for (const auto& od : ents)
            cc += std::min<size_t>(std::max<size_t>((size_t)S * od.H * od.nw * 32 / 64, 1024), 1u << 28);
        cap_cand = (uint32_t)std::min<size_t>(cc, 1u << 30);
        cap_ori = std::max(cap_ori, cap_cand);
        return ensure_lists();
    }

    int ensure_lists() {
        drop_graph();
        const size_t kp = sizeof(Keypoint);
        CK(d_cands.ensure((size_t)cap_cand * kp), "cudaMalloc(cands)");
        CK(d_refined.ensure((size_t)cap_cand * kp), "cudaMalloc(refined)");
        CK(d_keep.ensure((size_t)cap_cand * 4), "cudaMalloc(keep)");
        CK(d_ori_angle.ensure((size_t)cap_cand * kOriMaxPeaks * 4), "cudaMalloc(ori_angle)");
        CK(d_ori_count.ensure((size_t)cap_cand * 4), "cudaMalloc(ori_count)");
        CK(d_ori_off.ensure((size_t)cap_cand * 4), "cudaMalloc(ori_off)");
        CK(d_oriented.ensure((size_t)cap_ori * kp), "cudaMalloc(oriented)");
        CK(d_desc.ensure((size_t)cap_ori * kDescLen * 4), "cudaMalloc(desc)");
        scan_b = scan_state_words((size_t)std::max<long long>(total_words, 1));
        scan_words = scan_b + scan_state_words(cap_cand);
        CK(d_scan.ensure(scan_words * sizeof(unsigned long long)), "cudaMalloc(scan state)");
        return 0;
    }

    // Mapped export buffer for at least n keypoints of this batch geometry.
    int ensure_export(uint32_t n, bool geometry_changed) {
        if (hx.p && n <= cap_x && !geometry_changed) return 0;
        drop_graph();
        cap_x = std::max<uint32_t>(std::max<uint32_t>(2 * n + 4096, cap_x), 4096);
        hx.release();
        void* ptr = nullptr;
        const size_t bytes = hx_desc_off() + sizeof(float) * kDescLen * (size_t)cap_x;
        CK(cudaHostAlloc(&ptr, bytes, cudaHostAllocMapped), "cudaHostAlloc(batch export)");
        hx.p = ptr;
        hx.bytes = bytes;
        char* dptr = nullptr;
        CK(cudaHostGetDevicePointer((void**)&dptr, ptr, 0), "cudaHostGetDevicePointer");
        hx_dctr = reinterpret_cast<Counters*>(dptr);
        hx_dranges = reinterpret_cast<uint32_t*>(dptr + hx_ranges_off());
        hx_dkps = reinterpret_cast<Keypoint*>(dptr + hx_kps_off());
        hx_ddesc = reinterpret_cast<float*>(dptr + hx_desc_off());
        return 0;
    }

    // The whole batch after its images are in d_img.
    int enqueue() {
        const float* wts = d_wts.as<float>();
        const float* lut = wts + lut_off;
        uint8_t* U = d_U.as<uint8_t>();
        Counters* ctr = d_ctr.as<Counters>();
        OctCounters* oc = &ctr->oct[0];
        const BatchPyr bp = bpyr();
        const EntryTable tb = tab();
        int nl = 0;
        launches = 0;
        auto bump = [&](int rc, const char* what) -> int {
            if (rc) return cuda_fail(cudaGetLastError(), what);
            return 0;
        };
        CK(cudaMemsetAsync(d_ctr.p, 0, sizeof(Counters), st), "memset counters");
        CK(cudaMemsetAsync(d_scan.p, 0, scan_words * sizeof(unsigned long long), st), "memset scan state");
        auto level = [&](int o, int s, cudaStream_t q, uint8_t* tmp) -> int {
            const LevelBlur& b = s == 0 ? base : lv[o][s - 1];
            const OctPref& pf = opref[o];
            if (b.sigma <= 0.0f) {
                // a copy of the previous level (or of the image), image by image
                for (int i = 0; i < N; ++i) {
                    const OctaveDev& od = ents[(size_t)i * O + o];
                    if (od.W == 0 || od.H == 0) continue;
                    const uint8_t* src = s == 0 ? d_img.as<uint8_t>() + img_off[i] : U + od.u_off + (long long)(s - 1) * od.plane;
                    const size_t sp = s == 0 ? (size_t)img_pitch[i] : (size_t)od.pitch;
                    CK(cudaMemcpy2DAsync(U + od.u_off + (long long)s * od.plane, od.pitch, src, sp, od.W, od.H,
                                         cudaMemcpyDeviceToDevice, q),
                       "copy level");
                }
                return 0;
            }
            return bump(launch_blur_level_flat(bp, tmp, o, s, b.radius, N, pref(pf.fused), pf.n_fused, pref(pf.rows),
                                               pf.n_rows, max_w, pref(pf.cols), pf.n_cols, wts + b.woff, lut, q,
                                               &nl, 8),
                        "batch blur");
        };
        // pyramid
        if (int rc = level(0, 0, st, d_tmp.as<uint8_t>())) return rc;
        for (int o = 0; o < O; ++o) {
            for (int s = 1; s <= S; ++s)
                if (int rc = level(o, s, st, d_tmp.as<uint8_t>())) return rc;
            CK(cudaEventRecord(ev_lvl[o], st), "event record");
            CK(cudaStreamWaitEvent(st2, ev_lvl[o], 0), "stream wait");
            for (int s = S + 1; s < S + 3; ++s)
                if (int rc = level(o, s, st2, d_tmp2.as<uint8_t>())) return rc;
            if (o + 1 < O && opref[o].n_lz) {
                if (int rc = bump(launch_lanczos_flat(bp, o, N, pref(opref[o].lz), opref[o].n_lz, d_lz.p,
                                                      d_ltab.as<int>(), d_lw.as<float>(), st),
                                  "batch lanczos"))
                    return rc;
                ++nl;
            }
        }
        CK(cudaEventRecord(ev_side, st2), "event record");
        CK(cudaStreamWaitEvent(st, ev_side, 0), "stream wait");
        // detection over every entry
        unsigned long long* sst = d_scan.as<unsigned long long>();
        if (int rc = bump(launch_extrema_mask_flat(U, lut, tb, 0, N * O, pref(ex_pref), n_ex, (int)p.image_border_width,
                                                   d_words.as<uint32_t>(), st),
                          "batch extrema"))
            return rc;
        if (scan_exclusive(d_words.as<uint32_t>(), SCAN_POPC, d_cand_off.as<uint32_t>(), (size_t)total_words, nullptr,
                           &oc->n_cand, sst, &ctr->overflow, st))
            return cuda_fail(cudaGetLastError(), "batch scan");
        if (int rc = bump(launch_emit(U, lut, tb, 0, N * O, total_words, d_words.as<uint32_t>(),
                                      d_cand_off.as<uint32_t>(), d_cands.as<Keypoint>(), cap_cand, ctr, st),
                          "batch emit"))
            return rc;
        if (int rc = bump(launch_refine(U, lut, tb, p.sigma, p.contrast_threshold, p.edge_threshold,
                                        d_cands.as<Keypoint>(), d_refined.as<Keypoint>(), d_keep.as<uint32_t>(),
                                        cap_cand, oc, st),
                          "batch refine"))
            return rc;
        const int ogrid = (int)std::max<uint32_t>(cap_cand / 64, 32);
        if (int rc = bump(launch_orientation<uint8_t>(U, tb, lut, d_refined.as<Keypoint>(), d_keep.as<uint32_t>(),
                                                      cap_cand, oc, d_ori_angle.as<float>(), d_ori_count.as<uint32_t>(),
                                                      ogrid, 152 * 4, st),
                          "batch orientation"))
            return rc;
        if (scan_exclusive(d_ori_count.as<uint32_t>(), SCAN_U32, d_ori_off.as<uint32_t>(), cap_cand, &oc->n_cand,
                           &oc->n_ori, sst + scan_b, &ctr->overflow, st))
            return cuda_fail(cudaGetLastError(), "batch orientation scan");
        if (int rc = bump(launch_orient_emit(d_refined.as<Keypoint>(), cap_cand, 0, ctr, d_ori_angle.as<float>(),
                                             d_ori_count.as<uint32_t>(), d_ori_off.as<uint32_t>(),
                                             d_oriented.as<Keypoint>(), cap_ori, st),
                          "batch orientation emit"))
            return rc;
        const int dgrid = (int)std::max<uint32_t>(cap_cand / 16, 64);
        if (int rc = bump(launch_descriptor<uint8_t>(U, tb, d_oriented.as<Keypoint>(), oc, d_desc.as<float>(),
                                                     cap_ori, hx_ddesc, cap_x, dgrid, 152 * 8, st),
                          "batch descriptor"))
            return rc;
        if (launch_chained(k_batch_export, 152 * 4, 256, 0, st, d_ents.as<OctaveDev>(), O, N, total_words,
                           (const uint32_t*)d_cand_off.as<uint32_t>(), (const uint32_t*)d_ori_off.as<uint32_t>(),
                           (const Counters*)ctr, cap_cand, d_oriented.as<Keypoint>(), cap_ori, hx_dctr, hx_dranges,
                           hx_dkps, cap_x) != cudaSuccess)
            return cuda_fail(cudaGetLastError(), "batch export");
        launches = (uint32_t)nl + 11;  // extrema, 2 scans, emit, refine, orientation, its emit, descriptors, export
        return 0;
    }

    int run() {
        if (!gexec) {
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
            int rc = enqueue();
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return cuda_fail(e, "end capture");
            graph = g;
            CK(cudaGraphInstantiate(&gexec, graph, 0), "graph instantiate");
            graph_launches = launches;
        }
        launches = graph_launches;
        CK(cudaEventRecord(ev_t0, st), "event record");
        CK(cudaGraphLaunch(gexec, st), "graph launch");
        CK(cudaEventRecord(ev_t1, st), "event record");
        return 0;
    }

    int detect(const SiftCudaImage* imgs, uint32_t n) {
        CK(cudaSetDevice(opt.device), "cudaSetDevice");
        std::vector<std::pair<uint32_t, uint32_t>> d(n);
        for (uint32_t i = 0; i < n; ++i) {
            if ((!imgs[i].data && imgs[i].width && imgs[i].height) || imgs[i].stride < imgs[i].width)
                return fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "batch image: NULL data or stride < width");
            d[i] = {imgs[i].width, imgs[i].height};
        }
        const bool changed = ents.empty() || d != dims;
        if (int rc = ensure_geometry(d)) return rc;
        if (int rc = ensure_export(n_out, changed)) return rc;
        // The base level reads each image where it is: the caller's buffer on
        // a device that reads pageable host memory coherently, when every
        // image starts and strides on 16 bytes (the level kernel's staging
        // loads) and the base level is a blur (a copied base level is a copy
        // node that reads the device copy); else the batch's device copy.
        bool direct = host_reads && base.sigma > 0.0f;
        for (uint32_t i = 0; i < n && direct; ++i)
            if (imgs[i].width && imgs[i].height &&
                (((uintptr_t)imgs[i].data & 15) != 0 || (imgs[i].stride & 15) != 0 || imgs[i].stride > (1u << 30)))
                direct = false;
        h_addr.assign(n, 0);
        h_pitch.assign(n, 0);
        for (uint32_t i = 0; i < n; ++i) {
            if (direct) {
                h_addr[i] = (unsigned long long)(uintptr_t)imgs[i].data;
                h_pitch[i] = (int)imgs[i].stride;
            } else {
                h_addr[i] = (unsigned long long)(uintptr_t)(d_img.as<uint8_t>() + img_off[i]);
                h_pitch[i] = img_pitch[i];
                if (imgs[i].width && imgs[i].height)
                    CK(cudaMemcpy2DAsync(d_img.as<uint8_t>() + img_off[i], img_pitch[i], imgs[i].data,
                                         imgs[i].stride, imgs[i].width, imgs[i].height, cudaMemcpyHostToDevice, st),
                       "copy image");
            }
        }
        CK(cudaMemcpyAsync(d_imgaddr.p, h_addr.data(), sizeof(unsigned long long) * n, cudaMemcpyHostToDevice, st),
           "H2D image table");
        CK(cudaMemcpyAsync(d_imgpitch.p, h_pitch.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st),
           "H2D image table");
        images_in_place = direct;
        for (int attempt = 0; attempt < 8; ++attempt) {
            if (int rc = run()) return rc;
            CK(cudaStreamSynchronize(st), "batch run");
            CK(cudaEventElapsedTime(&device_ms, ev_t0, ev_t1), "event time");
            const Counters c = *hx.as<Counters>();
            if (c.overflow & 8u) return fail(SIFT_CUDA_ERR_CUDA, "a prefix-scan wait ran out (the run was abandoned)");
            bool grow = false;
            if (c.oct[0].n_cand > cap_cand || (c.overflow & 1u)) {
                const size_t nc = (size_t)c.oct[0].n_cand + c.oct[0].n_cand / 4 + 1024;
                if (nc > (1u << 30)) return fail(SIFT_CUDA_ERR_CAPACITY, "candidate list above 2^30");
                cap_cand = (uint32_t)nc;
                cap_ori = std::max(cap_ori, cap_cand);
                grow = true;
            }
            if (c.oct[0].n_ori > cap_ori || c.n_oriented > cap_ori || (c.overflow & 4u)) {
                const uint32_t no = std::max(c.oct[0].n_ori, c.n_oriented);
                const size_t nn = std::max<size_t>((size_t)cap_ori * 2, (size_t)no + no / 4 + 1024);
                if (nn > (1u << 30)) return fail(SIFT_CUDA_ERR_CAPACITY, "keypoint list above 2^30");
                cap_ori = (uint32_t)nn;
                grow = true;
            }
            if (grow) {
                if (int rc = ensure_lists()) return rc;
                continue;
            }
            if (c.oct[0].n_ori > cap_x) {  // more keypoints than the export buffer holds: grow it, run again
                if (int rc = ensure_export(c.oct[0].n_ori, false)) return rc;
                continue;
            }
            n_out = c.oct[0].n_ori;
            return 0;
        }
        return fail(SIFT_CUDA_ERR_CAPACITY, "keypoint lists kept overflowing");
    }
};

}  // namespace sift

struct SiftCudaBatch {
    sift::BatchEngine b;
};

extern "C" int sift_cuda_batch_create(const SiftCudaParams* params, const SiftCudaOptions* opts, SiftCudaBatch** out) {
    sift::g_last_error.clear();
    if (!params || !out) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "params or out is NULL");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return sift::fail(SIFT_CUDA_ERR_NO_DEVICE, "no CUDA device");
    SiftCudaOptions o;
    sift_cuda_options_default(&o);
    if (opts) o = *opts;
    if (o.storage != SIFT_CUDA_STORAGE_U8)
        return sift::fail(SIFT_CUDA_ERR_UNSUPPORTED, "the batched form keeps its levels as u8 planes (storage U8)");
    if (params->num_intervals < 1 || params->num_octaves < 1)
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "num_octaves and num_intervals must be >= 1");
    SiftCudaBatch* h = new (std::nothrow) SiftCudaBatch();
    if (!h) return sift::fail(SIFT_CUDA_ERR_OUT_OF_MEMORY, "host allocation");
    h->b.p = *params;
    h->b.opt = o;
    if (int rc = h->b.init()) {
        delete h;
        return rc;
    }
    *out = h;
    return 0;
}

extern "C" void sift_cuda_batch_destroy(SiftCudaBatch* batch) {
    if (!batch) return;
    cudaSetDevice(batch->b.opt.device);
    cudaStreamSynchronize(batch->b.st);
    delete batch;
}

extern "C" int sift_cuda_batch_detect_and_compute(SiftCudaBatch* batch, const SiftCudaImage* images, uint32_t n,
                                                  SiftCudaBatchResult* out) {
    sift::g_last_error.clear();
    if (!batch || !out || (n && !images)) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out, 0, sizeof *out);
    if (n == 0) return 0;
    sift::BatchEngine& b = batch->b;
    if (int rc = b.detect(images, n)) return rc;
    out->n_images = n;
    out->total = b.n_out;
    out->offsets = reinterpret_cast<const uint32_t*>(b.hx.as<char>() + b.hx_ranges_off());
    out->kps = reinterpret_cast<const SiftCudaKeypoint*>(b.hx.as<char>() + b.hx_kps_off());
    out->desc = reinterpret_cast<const float*>(b.hx.as<char>() + b.hx_desc_off());
    out->launches = b.launches;
    out->device_ms = b.device_ms;
    out->images_in_place = b.images_in_place ? 1u : 0u;
    return 0;
}
