// usct_engine.cu -- host side of the batched engine behind the C ABI in
// include/usct_gb300.h: plans, workspace carving, the checkpointed time loops
// and the small gather/prepare kernels.
//
// Time loops (one launch per time step for all C shots of a batch):
//   forward   n = 1..nt-1: p^n from (p^{n-1}, p^{n-2}) in two ping-pong
//             buffers; receivers sampled into slot rows; the pair
//             (p^{a-1}, p^a) copied out at every segment start a = j*k; the
//             last segment's d2p written straight into the stash.
//   backward  segments j = nseg-1..0: recompute levels a+1..b from the stored
//             pair with the same kernel (bit-identical), stashing d2p; then
//             adjoint steps k = b..a+1 consuming the stash (fwi.py:310-330).
// Memory per batch (levels of nz*ny*nxs*C floats): 2 state + 2*nseg
// checkpoints + k stash + 2 adjoint (+2 Born), see usct_batch_bytes.
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "usct_convert.cuh"
#include "usct_gb300.h"
#include "usct_kernels.cuh"
#include "usct_tma.cuh"
#include "usct_tma2.cuh"

namespace {
// NVTX range around an entry point (visible in Nsight timelines; a no-op
// when no tool is attached)
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};
}  // namespace

using namespace usct;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_err;

static int set_err(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CUDA_TRY(x)                                                                     \
    do {                                                                                \
        cudaError_t e_ = (x);                                                           \
        if (e_ != cudaSuccess)                                                          \
            return set_err(e_ == cudaErrorMemoryAllocation ? USCT_ERR_NOMEM : USCT_ERR_CUDA, \
                           "%s: %s", #x, cudaGetErrorString(e_));                       \
    } while (0)

#define TRY(x)                   \
    do {                         \
        int r_ = (x);            \
        if (r_ != USCT_OK) return r_; \
    } while (0)

extern "C" const char* usct_last_error(void) { return g_err.c_str(); }

// Error reporting for the other translation units of the library.
int usct_internal_error(int code, const char* msg) {
    g_err = msg ? msg : "";
    return code;
}
extern "C" int usct_version(void) { return 10000; }

// ---------------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------------
struct usct_plan {
    int device = 0;
    int ndim = 0;
    int dims[3] = {0, 0, 0};
    double h = 0, dt = 0;
    int nt = 0, n_tx = 0, n_rx = 0;
    Geo geo{};
    int txv = 0, ty = 0, nzc = 0, ntx_t = 0, nty_t = 0, ntiles = 0;
    int C = 0, logC = 0, nbatch = 0, k = 0, nseg = 0;
    size_t N = 0, cells_p = 0, LV = 0;
    int nslot = 0;
    int* d_sptr = nullptr;
    SrcEnt* d_sent = nullptr;
    int* d_rptr = nullptr;
    RxEnt* d_rent = nullptr;
    int* d_rxptr = nullptr;
    // plain one-shot form (point elements): cells and weights per transmit/receiver
    std::vector<int> h_tx_ptr, h_rx_ptr;
    std::vector<int64_t> h_tx_cell, h_rx_cell;
    std::vector<double> h_tx_w, h_rx_w;
    int64_t* d_tx_cell = nullptr;
    float* d_tx_w = nullptr;
    int64_t* d_rx_cell = nullptr;
    bool has_sp = false, has_vm = false;
    long long launches = 0;
    // kernel variant: 0 = register-queue stencils, 1 = TMA-fed shared-memory ring
    int variant = 0;
    int stages_fwd = 4, stages_born = 3, stages_adj = 4;
    // two time levels per forward launch (usct_tma2.cuh): tile w2 x h2 cells,
    // its own tiling (ntx2 x nty2 tiles, nzc2 chunks of zc2 planes), ring
    // depths and per-tile lists (sources of the tile grown by one cell/row)
    int tb = 0, w2 = 0, h2 = 0, zc2 = 0, zc2_req = 0, ntx2 = 0, nty2 = 0, nzc2 = 0, ntiles2 = 0;
    int ra2 = 5, rb2 = 4;
    int* d_sptr2 = nullptr;
    SrcEnt* d_sent2 = nullptr;
    int* d_rptr2 = nullptr;
    RxEnt* d_rent2 = nullptr;
    // every shot channel on its own model (co-admitted requests in one launch):
    // transmit t uses model d_tx_model[t] of n_models
    int pcs = 0, n_models = 0;
    int* d_tx_model = nullptr;
    int* d_err = nullptr;   // set by a kernel whose bounded wait gave up
    std::unordered_map<uint64_t, CUtensorMap> maps;
    // CUDA graphs of whole batch sweeps, keyed by (op, batch, mode, buffers)
    bool use_graphs = false;
    int wait_test = 0;   // USCT_SET_WAIT_TEST
    struct Captured {
        cudaGraphExec_t exec;
        long long kernels;
    };
    std::map<std::tuple<int, int, int, const void*, const void*, const void*>, Captured> graphs;
};

static void drop_graphs(usct_plan* p) {
    for (auto& kv : p->graphs) cudaGraphExecDestroy(kv.second.exec);
    p->graphs.clear();
}

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }
static int ilog2(int c) { int l = 0; while ((1 << l) < c) ++l; return l; }
static bool pow2(int c) { return c > 0 && (c & (c - 1)) == 0; }

static bool tile_supported(bool is3d, int txv, int ty) {
    if (is3d) return (txv == 32 && (ty == 4 || ty == 8)) || (txv == 64 && (ty == 2 || ty == 4));
    return ty == 1 && (txv == 64 || txv == 128);
}

// The TMA ring needs 16-byte rows in every box: a tile row must hold at least
// 4 cells of the model (TXF >= 4C), and for batches narrower than 4 shots
// (boxes of whole rows) the row box must fit 256 elements (tile_x == 32, 3D).
static void init_tma_attributes();

static bool tma_supported(const usct_plan* p) { return tma_tile_ok(p->txv, p->C, p->ndim == 3); }

// two time levels per forward launch: the default tile per batch width, the
// tiles there are kernels for, and the shared memory of a launch
static int tb_default_tile(int C) { return C >= 64 ? 408 : (C >= 32 ? 808 : 1608); }
static bool tb_tile_ok(int key) {
    return key == 408 || key == 804 || key == 808 || key == 1604 || key == 1608;
}
static bool tb_on(const usct_plan* p) { return p->tb && p->variant == 1; }

static size_t tb_smem(const usct_plan* p, bool has_sp) {
    const Fwd2Layout L = fwd2_layout(p->w2, p->h2, p->C, has_sp, p->ra2, p->rb2);
    return (size_t)L.floats * sizeof(float) + (size_t)(p->ra2 + p->rb2) * 8 + 16;
}


static void free_tb_lists(usct_plan* p) {
    cudaFree(p->d_sptr2); cudaFree(p->d_sent2); cudaFree(p->d_rptr2); cudaFree(p->d_rent2);
    p->d_sptr2 = nullptr; p->d_sent2 = nullptr; p->d_rptr2 = nullptr; p->d_rent2 = nullptr;
}

static void free_plan_dev(usct_plan* p) {
    free_tb_lists(p);
    cudaFree(p->d_tx_model);
    p->d_tx_model = nullptr;
    cudaFree(p->d_sptr); cudaFree(p->d_sent); cudaFree(p->d_rptr); cudaFree(p->d_rent);
    cudaFree(p->d_rxptr); cudaFree(p->d_tx_cell); cudaFree(p->d_tx_w); cudaFree(p->d_rx_cell);
    cudaFree(p->d_err);
    p->d_err = nullptr;
    p->d_sptr = nullptr; p->d_sent = nullptr; p->d_rptr = nullptr; p->d_rent = nullptr;
    p->d_rxptr = nullptr; p->d_tx_cell = nullptr; p->d_tx_w = nullptr; p->d_rx_cell = nullptr;
}

template <class T>
static int upload(T** dst, const std::vector<T>& v) {
    const size_t n = std::max<size_t>(v.size(), 1);
    CUDA_TRY(cudaMalloc(dst, n * sizeof(T)));
    if (!v.empty()) CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return USCT_OK;
}

static int check_csr(const char* what, int n, const int* ptr, const int64_t* cell, const double* w,
                     int64_t ncell) {
    if (!ptr) return set_err(USCT_ERR_ARG, "%s: null pointer array", what);
    if (ptr[0] != 0) return set_err(USCT_ERR_ARG, "%s: ptr[0] must be 0", what);
    for (int i = 0; i < n; ++i)
        if (ptr[i + 1] < ptr[i]) return set_err(USCT_ERR_ARG, "%s: ptr not monotone at %d", what, i);
    const int ne = ptr[n];
    if (ne > 0 && (!cell || !w)) return set_err(USCT_ERR_ARG, "%s: null cell/weight array", what);
    for (int e = 0; e < ne; ++e) {
        if (cell[e] < 0 || cell[e] >= ncell)
            return set_err(USCT_ERR_ARG, "%s: cell %lld of entry %d outside the grid (%lld cells)",
                           what, (long long)cell[e], e, (long long)ncell);
        if (!std::isfinite(w[e])) return set_err(USCT_ERR_ARG, "%s: non-finite weight at %d", what, e);
    }
    return USCT_OK;
}

// cell -> (z, y, x) in the engine's axis convention (2D: z = row, y = 0)
static void unravel(const usct_plan* p, int64_t cell, int& z, int& y, int& x) {
    const int nx = p->geo.nx, ny = p->geo.ny;
    x = (int)(cell % nx);
    const int64_t r = cell / nx;
    y = (int)(r % ny);
    z = (int)(r / ny);
}

extern "C" int usct_plan_create(usct_plan** out, int ndim, const int* dims, double h, double dt,
                                int nt, int n_tx, const int* tx_ptr, const int64_t* tx_cell,
                                const double* tx_w, int n_rx, const int* rx_ptr,
                                const int64_t* rx_cell, const double* rx_w, int batch, int ckpt_k,
                                int tile_x, int tile_y, int zchunk) {
    if (!out) return set_err(USCT_ERR_ARG, "out is null");
    *out = nullptr;
    if (ndim != 2 && ndim != 3) return set_err(USCT_ERR_ARG, "ndim must be 2 or 3 (got %d)", ndim);
    if (!dims) return set_err(USCT_ERR_ARG, "dims is null");
    for (int d = 0; d < ndim; ++d)
        if (dims[d] < 3) return set_err(USCT_ERR_ARG, "dims[%d] = %d < 3", d, dims[d]);
    if (nt < 2) return set_err(USCT_ERR_ARG, "nt must be >= 2 (got %d)", nt);
    if (!(h > 0) || !(dt > 0)) return set_err(USCT_ERR_ARG, "h and dt must be positive");
    if (n_tx < 1 || n_rx < 1) return set_err(USCT_ERR_ARG, "need at least one transmit and one receiver");
    if (batch != 0 && (!pow2(batch) || batch > 64))
        return set_err(USCT_ERR_ARG, "batch must be a power of two <= 64 (got %d)", batch);
    if (ckpt_k != 0 && ckpt_k < 2) return set_err(USCT_ERR_ARG, "ckpt_k must be >= 2 (got %d)", ckpt_k);

    usct_plan* p = new usct_plan();
    cudaGetDevice(&p->device);
    p->ndim = ndim;
    for (int d = 0; d < ndim; ++d) p->dims[d] = dims[d];
    p->h = h; p->dt = dt; p->nt = nt; p->n_tx = n_tx; p->n_rx = n_rx;
    Geo& g = p->geo;
    if (ndim == 3) { g.nz = dims[0]; g.ny = dims[1]; g.nx = dims[2]; }
    else { g.nz = dims[0]; g.ny = 1; g.nx = dims[1]; }
    p->N = (size_t)g.nz * g.ny * g.nx;
    int ret = check_csr("sources", n_tx, tx_ptr, tx_cell, tx_w, (int64_t)p->N);
    if (ret == USCT_OK) ret = check_csr("receivers", n_rx, rx_ptr, rx_cell, rx_w, (int64_t)p->N);
    if (ret != USCT_OK) { delete p; return ret; }

    int C = batch;
    if (C == 0) { C = 1; while (C < n_tx && C < 32) C <<= 1; }
    p->C = C; p->logC = ilog2(C);
    p->nbatch = (n_tx + C - 1) / C;
    g.C = C; g.logC = p->logC;
    g.nxs = (g.nx + 3) & ~3;
    g.RP = g.nxs * C;
    g.PP = (long long)g.RP * g.ny;
    g.CPP = (long long)g.nxs * g.ny;
    g.inv_h2 = (float)(1.0 / (h * h));
    p->cells_p = (size_t)g.CPP * g.nz;
    p->LV = (size_t)g.PP * g.nz;

    const bool is3d = ndim == 3;
    int txv = tile_x, ty = tile_y;
    if (txv == 0) txv = is3d ? (C >= 16 ? 64 : 32) : 128;
    if (ty == 0 || !is3d) ty = is3d ? (txv == 64 ? 4 : 8) : 1;
    if (!tile_supported(is3d, txv, ty)) {
        delete p;
        return set_err(USCT_ERR_ARG, "unsupported tile %dx%d for %dD", txv, ty, ndim);
    }
    if (4 * txv < C) { delete p; return set_err(USCT_ERR_ARG, "tile row narrower than the batch"); }
    p->txv = txv; p->ty = ty;
    p->ntx_t = (g.RP + 4 * txv - 1) / (4 * txv);
    p->nty_t = (g.ny + ty - 1) / ty;
    p->ntiles = p->ntx_t * p->nty_t;
    g.ntiles_x = p->ntx_t;
    int zc = zchunk;
    if (zc <= 0) {
        const long long target = 152LL * 16;   // CTAs for a few full waves
        long long nzc = (target + p->ntiles - 1) / p->ntiles;
        nzc = std::max<long long>(1, std::min<long long>(nzc, g.nz / 8 > 0 ? g.nz / 8 : 1));
        zc = (int)((g.nz + nzc - 1) / nzc);
    }
    zc = std::max(1, std::min(zc, g.nz));
    g.zc = zc;
    p->nzc = (g.nz + zc - 1) / zc;
    if (p->nty_t > 65535 || p->nzc > 65535) { delete p; return set_err(USCT_ERR_ARG, "grid too large"); }

    int k = ckpt_k;
    if (k == 0) {
        k = (int)std::lround(std::sqrt(2.0 * (nt - 1)));
        k = std::max(2, k);
    }
    k = std::min(k, std::max(2, nt - 1));
    p->k = k;
    p->nseg = (nt - 1 + k - 1) / k;

    // plain-form copies
    p->h_tx_ptr.assign(tx_ptr, tx_ptr + n_tx + 1);
    p->h_rx_ptr.assign(rx_ptr, rx_ptr + n_rx + 1);
    p->h_tx_cell.assign(tx_cell, tx_cell + tx_ptr[n_tx]);
    p->h_rx_cell.assign(rx_cell, rx_cell + rx_ptr[n_rx]);
    p->h_tx_w.assign(tx_w, tx_w + tx_ptr[n_tx]);
    p->h_rx_w.assign(rx_w, rx_w + rx_ptr[n_rx]);

    // per-tile source entries, per batch
    const int TXF = 4 * txv, cpt = TXF / C;   // cells per tile row
    std::vector<int> sptr((size_t)p->nbatch * (p->ntiles + 1), 0);
    std::vector<SrcEnt> sent;
    for (int b = 0; b < p->nbatch; ++b) {
        std::vector<std::pair<int, SrcEnt>> tmp;   // (tile, entry)
        for (int c = 0; c < C; ++c) {
            const int t = b * C + c;
            if (t >= n_tx) break;
            for (int e = tx_ptr[t]; e < tx_ptr[t + 1]; ++e) {
                int z, y, x;
                unravel(p, tx_cell[e], z, y, x);
                const int xt = x / cpt, yt = y / ty;
                SrcEnt se{z, y - yt * ty, (x - xt * cpt) * C + c, (float)tx_w[e]};
                tmp.push_back({xt + p->ntx_t * yt, se});
            }
        }
        std::stable_sort(tmp.begin(), tmp.end(), [](const auto& a, const auto& b2) {
            return a.first != b2.first ? a.first < b2.first : a.second.z < b2.second.z;
        });
        int* bp = &sptr[(size_t)b * (p->ntiles + 1)];
        const int base = (int)sent.size();
        size_t q = 0;
        for (int tl = 0; tl < p->ntiles; ++tl) {
            bp[tl] = base + (int)q;
            while (q < tmp.size() && tmp[q].first == tl) { sent.push_back(tmp[q].second); ++q; }
        }
        bp[p->ntiles] = base + (int)q;
    }
    // per-tile receiver entries (shared by all batches), ordered (z, ly, lcell, j)
    std::vector<std::pair<int, RxEnt>> rtmp;
    for (int j = 0; j < n_rx; ++j)
        for (int e = rx_ptr[j]; e < rx_ptr[j + 1]; ++e) {
            int z, y, x;
            unravel(p, rx_cell[e], z, y, x);
            const int xt = x / cpt, yt = y / ty;
            RxEnt re{z, y - yt * ty, x - xt * cpt, e, j, (float)rx_w[e], 0, 0};
            rtmp.push_back({xt + p->ntx_t * yt, re});
        }
    std::stable_sort(rtmp.begin(), rtmp.end(), [](const auto& a, const auto& b2) {
        if (a.first != b2.first) return a.first < b2.first;
        if (a.second.z != b2.second.z) return a.second.z < b2.second.z;
        if (a.second.ly != b2.second.ly) return a.second.ly < b2.second.ly;
        return a.second.lcell < b2.second.lcell;
    });
    std::vector<int> rptr(p->ntiles + 1, 0);
    std::vector<RxEnt> rent;
    {
        size_t q = 0;
        for (int tl = 0; tl < p->ntiles; ++tl) {
            rptr[tl] = (int)q;
            while (q < rtmp.size() && rtmp[q].first == tl) { rent.push_back(rtmp[q].second); ++q; }
        }
        rptr[p->ntiles] = (int)q;
    }
    p->nslot = rx_ptr[n_rx];
    std::vector<int> rxptr(rx_ptr, rx_ptr + n_rx + 1);
    std::vector<float> txwf(p->h_tx_w.begin(), p->h_tx_w.end());

    if ((ret = upload(&p->d_sptr, sptr)) != USCT_OK || (ret = upload(&p->d_sent, sent)) != USCT_OK ||
        (ret = upload(&p->d_rptr, rptr)) != USCT_OK || (ret = upload(&p->d_rent, rent)) != USCT_OK ||
        (ret = upload(&p->d_rxptr, rxptr)) != USCT_OK ||
        (ret = upload(&p->d_tx_cell, p->h_tx_cell)) != USCT_OK ||
        (ret = upload(&p->d_tx_w, txwf)) != USCT_OK ||
        (ret = upload(&p->d_rx_cell, p->h_rx_cell)) != USCT_OK ||
        (ret = upload(&p->d_err, std::vector<int>(1, 0))) != USCT_OK) {
        free_plan_dev(p);
        delete p;
        return ret;
    }
    p->variant = tma_supported(p) ? 1 : 0;
    // 3D forward sweeps keep six planes in flight and Born sweeps five
    // (measured best at 192^3 / 320^3, and for the 224^3 Gauss-Newton product);
    // the 2D rows are short and four (three) suffice
    p->stages_fwd = ndim == 3 ? 6 : 4;
    p->stages_born = ndim == 3 ? 5 : 3;
    init_tma_attributes();
    *out = p;
    return USCT_OK;
}

extern "C" void usct_plan_destroy(usct_plan* p) {
    if (!p) return;
    drop_graphs(p);
    free_plan_dev(p);
    delete p;
}

extern "C" int usct_plan_info(const usct_plan* p, int key, int64_t* value) {
    if (!p || !value) return set_err(USCT_ERR_ARG, "null argument");
    switch (key) {
        case USCT_INFO_BATCH: *value = p->C; break;
        case USCT_INFO_NBATCH: *value = p->nbatch; break;
        case USCT_INFO_CKPT_K: *value = p->k; break;
        case USCT_INFO_NSEG: *value = p->nseg; break;
        case USCT_INFO_TILE_X: *value = p->txv; break;
        case USCT_INFO_TILE_Y: *value = p->ty; break;
        case USCT_INFO_ZCHUNK: *value = p->geo.zc; break;
        case USCT_INFO_LEVEL_FLOATS: *value = (int64_t)p->LV; break;
        case USCT_INFO_LAUNCHES: *value = p->launches; break;
        case USCT_INFO_VARIANT: *value = p->variant; break;
        case USCT_INFO_TBLOCK: *value = p->tb ? p->w2 * 100 + p->h2 : 0; break;
        default: return set_err(USCT_ERR_ARG, "unknown info key %d", key);
    }
    return USCT_OK;
}

// ---------------------------------------------------------------------------
// workspaces
// ---------------------------------------------------------------------------
struct ModelWS {
    float* S; float* sp; float* vm; float* wav; double* g;
    float* Spc;   // per-channel models: S of every batch, one value per four channels
};

// floats of one batch's per-channel S ([z][y][x][C/4], 256-byte aligned)
static size_t spc_floats(const usct_plan* p) {
    return al256(p->LV / 4 * sizeof(float)) / sizeof(float);
}
static const int JBLK = 64;   // gather blocks (per-block FP64 misfit partials)

static ModelWS carve_model(const usct_plan* p, void* base) {
    char* c = (char*)base;
    ModelWS m;
    const size_t cf = al256(p->cells_p * sizeof(float));
    m.S = (float*)c; c += cf;
    m.sp = (float*)c; c += cf;
    m.vm = (float*)c; c += cf;
    m.wav = (float*)c; c += al256((size_t)p->nt * sizeof(float));
    m.g = (double*)c; c += al256(p->cells_p * sizeof(double));
    m.Spc = p->pcs ? (float*)c : nullptr;
    return m;
}

extern "C" size_t usct_model_bytes(const usct_plan* p) {
    if (!p) return 0;
    return 3 * al256(p->cells_p * sizeof(float)) + al256((size_t)p->nt * sizeof(float)) +
           al256(p->cells_p * sizeof(double)) +
           (p->pcs ? (size_t)p->nbatch * spc_floats(p) * sizeof(float) : 0);
}

struct BatchWS {
    float* P[2]; float* rs; float* res; double* jpart; double* gj; float* ck; float* stash; float* L[2];
    float* D[2];
    float* P2[2];   // the second pair of state levels of two-step sweeps
};

static BatchWS carve_batch(const usct_plan* p, void* base, int mode) {
    char* c = (char*)base;
    BatchWS w{};
    const size_t lv = al256(p->LV * sizeof(float));
    w.P[0] = (float*)c; c += lv;
    w.P[1] = (float*)c; c += lv;
    w.rs = (float*)c; c += al256((size_t)p->nt * p->nslot * p->C * sizeof(float));
    w.res = (float*)c; c += al256((size_t)p->nt * p->n_rx * p->C * sizeof(float));
    w.jpart = (double*)c; c += al256((size_t)JBLK * p->C * sizeof(double));
    w.gj = (double*)c; c += al256((size_t)p->n_rx * p->C * sizeof(double));
    if (mode >= USCT_MODE_GRADIENT) {
        w.L[0] = (float*)c; c += lv;
        w.L[1] = (float*)c; c += lv;
        w.ck = (float*)c; c += (size_t)p->nseg * 2 * lv;
        w.stash = (float*)c; c += (size_t)p->k * lv;
    }
    if (mode == USCT_MODE_BORN) {
        w.D[0] = (float*)c; c += lv;
        w.D[1] = (float*)c; c += lv;
    }
    if (p->tb) {
        w.P2[0] = (float*)c; c += lv;
        w.P2[1] = (float*)c; c += lv;
    }
    return w;
}

extern "C" size_t usct_batch_bytes(const usct_plan* p, int mode) {
    if (!p || mode < 0 || mode > 2) return 0;
    const size_t lv = al256(p->LV * sizeof(float));
    size_t b = 2 * lv + al256((size_t)p->nt * p->nslot * p->C * sizeof(float)) +
               al256((size_t)p->nt * p->n_rx * p->C * sizeof(float)) +
               al256((size_t)JBLK * p->C * sizeof(double)) +
               al256((size_t)p->n_rx * p->C * sizeof(double));
    if (mode >= USCT_MODE_GRADIENT) b += (2 + 2 * (size_t)p->nseg + (size_t)p->k) * lv;
    if (mode == USCT_MODE_BORN) b += 2 * lv;
    if (p->tb) b += 2 * lv;
    return b;
}

// ---------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------
__global__ void k_prepare(const double* __restrict__ m, const double* __restrict__ sp,
                          const double* __restrict__ v, float* S, float* spo, float* vm, double dt2,
                          int nx, int nxs, long long ncp) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ncp;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % nxs);
        const long long r = i / nxs;
        if (x < nx) {
            const long long u = r * nx + x;
            const double mu = m[u];
            S[i] = (float)(dt2 / mu);
            spo[i] = sp ? (float)sp[u] : 1.f;
            vm[i] = v ? (float)(v[u] / mu) : 0.f;
        } else {
            S[i] = 0.f; spo[i] = 0.f; vm[i] = 0.f;
        }
    }
}

// One batch's S, [z][y][x][C/4], from per-transmit models: quad q of a cell
// holds channels 4q .. 4q+3, which share one model (usct_plan_set_channel_models
// checks it), so it takes the model of transmit 4q; quads past the batch's last
// transmit and padded cells get 0 (their fields stay 0).
__global__ void k_prepare_channels(const double* __restrict__ models, const int* __restrict__ tx_model,
                                   float* Spc, double dt2, int nx, int nxs, int C, int logC,
                                   int n_tx, long long ncp, long long total) {
    const int Q = C >> 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(i & (Q - 1));
        const long long cell = i >> (logC - 2);
        const int t = 4 * q;
        const int x = (int)(cell % nxs);
        float v = 0.f;
        if (t < n_tx && x < nx) {
            const long long u = (cell / nxs) * nx + x;
            v = (float)(dt2 / models[(long long)tx_model[t] * (ncp / nxs) * nx + u]);
        }
        Spc[i] = v;
    }
}

__global__ void k_wavelet(const double* __restrict__ w, float* o, int nt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nt) o[i] = (float)w[i];
}

__global__ void k_finalize(double* g, const double* __restrict__ m, double* grad, int nx, int nxs,
                           long long ncp) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ncp;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % nxs);
        const long long r = i / nxs;
        if (x < nx) {
            const long long u = r * nx + x;
            grad[u] = g[i] / m[u];
        }
        g[i] = 0.0;
    }
}

// Traces of receiver j = ordered sum of its slot samples (fwi.py:74-76); export
// to the user layout, and build the adjoint source: mode 1 r = tr - dobs with
// per-channel FP64 misfit partials, mode 2 r = tr (Born data), 0 none.
__global__ void __launch_bounds__(256) k_gather(const float* __restrict__ rs, int nslot, int C, int logC,
                                                int nt, int nrx, const int* __restrict__ rx_ptr,
                                                int shot0, int nb, float* out,
                                                const float* __restrict__ dobs, float* res,
                                                int mode, double* jpart,
                                                const float* __restrict__ tw) {
    __shared__ double sj[256];
    const int tid = threadIdx.x;
    const int c = tid & (C - 1);
    const int rstep = 256 >> logC;
    const long long rows = (long long)nt * nrx;
    const long long per = (rows + gridDim.x - 1) / gridDim.x;
    const long long r0 = blockIdx.x * per;
    const long long r1 = min(rows, r0 + per);
    double J = 0.0;
    for (long long r = r0 + (tid >> logC); r < r1; r += rstep) {
        const int n = (int)(r / nrx), j = (int)(r % nrx);
        float tr = 0.f;
        for (int e = rx_ptr[j]; e < rx_ptr[j + 1]; ++e) tr = tr + rs[((long long)n * nslot + e) * C + c];
        if (c < nb) {
            const long long uo = ((long long)(shot0 + c) * nt + n) * nrx + j;
            if (out) out[uo] = tr;
            if (mode == 1) {
                if (tw) {
                    // windowed data (fwi.py:298-301): r = dsyn W - dobs W, adjoint source r W
                    const float wv = tw[uo];
                    const float rr = tr * wv - dobs[uo] * wv;
                    res[r * C + c] = rr * wv;
                    J += 0.5 * (double)rr * (double)rr;
                } else {
                    const float rr = tr - dobs[uo];
                    res[r * C + c] = rr;
                    J += 0.5 * (double)rr * (double)rr;
                }
            } else if (mode == 2) {
                res[r * C + c] = tw ? tr * tw[uo] : tr;
            }
        } else if (mode) {
            res[r * C + c] = 0.f;
        }
    }
    sj[tid] = J;
    __syncthreads();
    for (int s = 128; s >= C && s > 0; s >>= 1) {
        if (tid < s) sj[tid] += sj[tid + s];
        __syncthreads();
    }
    if (jpart && tid < C) jpart[blockIdx.x * C + tid] = sj[tid];
}

__global__ void k_jsum(const double* __restrict__ jpart, int C, int nblk, int shot0, int nb, double* J) {
    const int c = threadIdx.x;
    if (c < nb) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += jpart[b * C + c];
        J[shot0 + c] = s;
    }
}

__global__ void k_adjsrc(const float* __restrict__ adj, float* res, int C, int nt, int nrx, int shot0,
                         int nb) {
    const long long tot = (long long)nt * nrx * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long r = i / C;
        const int n = (int)(r / nrx), j = (int)(r % nrx);
        res[i] = c < nb ? adj[((long long)(shot0 + c) * nt + n) * nrx + j] : 0.f;
    }
}

// GCN adjoint source (libuap.hpp:133-162, fwi.py:158-167) from the traces in
// res ([nt][n_rx][C]), in place, for each (receiver j, shot c):
//   sn = sqrt(sum sv^2) + eps, on = sqrt(sum ov^2) + eps,
//   c_j = sum sv*ov / (sn*on)   (= sum (sv/sn)(ov/on), the reference's form),
//   adj = a*ov + b*sv with a = -1/(on*sn), b = c_j/(sn*sn)
//         (= -(ov/on - c_j*sv/sn)/sn, the reference's form),
// and gj[j][c] = 1 - c_j for the per-shot misfit.  The sums are FP64 over the
// FP32 traces, each accumulated with fused multiply-adds over kGS contiguous
// time slices and the slices added in order -- no division per sample (the
// FP64 pipe is small on this part).  Block (32, kGS): lane x owns the trace
// idx = 32*blockIdx.x + x (idx = j*C + c), row y one time slice; the lanes of
// a warp read 32 consecutive floats of a time level.  With a window tw the
// traces in res are already windowed, dobs is windowed here and the adjoint
// source is multiplied by the window (fwi.py:298-301).
constexpr int kGS = 8;
__global__ void __launch_bounds__(32 * kGS) k_gcn(float* res, const float* __restrict__ dobs, int C,
                                                  int logC, int nt, int nrx, int shot0, int nb,
                                                  double* gj, const float* __restrict__ tw) {
    __shared__ double part[kGS][32][3];
    __shared__ double coef[32][2];
    const int x = threadIdx.x, y = threadIdx.y;
    const int idx = blockIdx.x * 32 + x;
    const bool live = idx < nrx * C;
    const int j = idx >> logC, c = idx & (C - 1);
    const bool shot = live && c < nb;
    const long long rstride = (long long)nrx * C;
    float* col = res + (long long)j * C + c;
    const int L = (nt + kGS - 1) / kGS;
    const int n0 = min(nt, y * L), n1 = min(nt, n0 + L);
    const float* ob = shot ? dobs + (long long)(shot0 + c) * nt * nrx + j : nullptr;
    const float* wb = (shot && tw) ? tw + (long long)(shot0 + c) * nt * nrx + j : nullptr;
    auto obs = [&](int n) -> double {
        const long long o = (long long)n * nrx;
        return usct_cvt::f32_to_f64(wb ? ob[o] * wb[o] : ob[o]);
    };
    double ss = 0.0, oo = 0.0, so = 0.0;
    if (shot) {
        for (int n = n0; n < n1; ++n) {
            const double sv = usct_cvt::f32_to_f64(col[n * rstride]);
            const double ov = obs(n);
            ss = fma(sv, sv, ss);
            oo = fma(ov, ov, oo);
            so = fma(sv, ov, so);
        }
    }
    part[y][x][0] = ss;
    part[y][x][1] = oo;
    part[y][x][2] = so;
    __syncthreads();
    if (y == 0 && live) {
        double S = 0.0, O = 0.0, D = 0.0;
        for (int q = 0; q < kGS; ++q) {
            S += part[q][x][0];
            O += part[q][x][1];
            D += part[q][x][2];
        }
        const double eps = 1e-12;
        const double sn = sqrt(S) + eps, on = sqrt(O) + eps;
        const double cc = D / (sn * on);
        coef[x][0] = -1.0 / (on * sn);
        coef[x][1] = cc / (sn * sn);
        gj[idx] = shot ? 1.0 - cc : 0.0;
    }
    __syncthreads();
    if (!live) return;
    if (!shot) {
        for (int n = n0; n < n1; ++n) col[n * rstride] = 0.f;
        return;
    }
    const double A = coef[x][0], B = coef[x][1];
    for (int n = n0; n < n1; ++n) {
        const double sv = usct_cvt::f32_to_f64(col[n * rstride]);
        const float adj = usct_cvt::f64_to_f32(fma(A, obs(n), B * sv));
        col[n * rstride] = wb ? adj * wb[(long long)n * nrx] : adj;
    }
}

__global__ void k_gcn_j(const double* __restrict__ gj, int C, int nrx, int shot0, int nb, double* J) {
    const int c = threadIdx.x;
    if (c < nb) {
        double s = 0.0;
        for (int j = 0; j < nrx; ++j) s += gj[(long long)j * C + c];
        J[shot0 + c] = s;
    }
}

// ---------------------------------------------------------------------------
// launches
// ---------------------------------------------------------------------------
static size_t stencil_smem(const usct_plan* p, int nfield) {
    const int HF = p->C < 4 ? 4 : p->C;
    return sizeof(float) * 2 * nfield * (p->ty + 2) * (4 * p->txv + 2 * HF);
}

// ---- tensor maps for the TMA ring -------------------------------------------
enum MapKind { MK_WF_HALO = 0, MK_WF_OWN = 1, MK_CELL_OWN = 2, MK_CELL_HALO = 3, MK_G_OWN = 4,
               MK2_A = 5, MK2_B = 6, MK2_S = 7,   // MK2_*: the two-step tiles
               MK_QUAD_OWN = 8 };                 // per-channel models: one S per 4 channels

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
    });
    return fn;
}

// Box shapes (innermost first).  Wavefields: 4D {C, nxs, ny, nz} when C >= 4,
// otherwise 3D {RP, ny, nz}; model cells: 3D {nxs, ny, nz} (float or double).
static int get_map(usct_plan* p, const void* ptr, int kind, CUtensorMap* out) {
    const uint64_t key = (uint64_t)(uintptr_t)ptr * 16u + (uint64_t)kind;
    auto it = p->maps.find(key);
    if (it != p->maps.end()) { *out = it->second; return USCT_OK; }
    auto enc = encode_fn();
    if (!enc) return set_err(USCT_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const Geo& g = p->geo;
    const int TXF = 4 * p->txv, cells = TXF >> g.logC, HR = p->ndim == 3 ? 1 : 0;
    const int rows_h = p->ty + 2 * HR;
    cuuint64_t dims[4] = {0, 0, 0, 0}, strides[3] = {0, 0, 0};
    cuuint32_t box[4] = {1, 1, 1, 1}, estr[4] = {1, 1, 1, 1};
    cuuint32_t rank = 3;
    CUtensorMapDataType dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const bool halo = kind == MK_WF_HALO;
    if (kind == MK2_A || kind == MK2_B) {
        // two-step tiles: p^{n-1} grown by two cells/rows, p^{n-2} by one
        const int grow = kind == MK2_A ? 4 : 2;
        rank = 4;
        dims[0] = g.C; dims[1] = g.nxs; dims[2] = g.ny; dims[3] = g.nz;
        strides[0] = (cuuint64_t)g.C * 4; strides[1] = (cuuint64_t)g.RP * 4;
        strides[2] = (cuuint64_t)g.PP * 4;
        box[0] = g.C; box[1] = p->w2 + grow; box[2] = p->h2 + grow; box[3] = 1;
    } else if (kind == MK2_S) {
        // S / sponge of the grown tile, 4 cells wider on each side so the
        // box's x coordinate stays 16-byte aligned
        dims[0] = g.nxs; dims[1] = g.ny; dims[2] = g.nz;
        strides[0] = (cuuint64_t)g.nxs * 4; strides[1] = (cuuint64_t)g.CPP * 4;
        box[0] = p->w2 + 8; box[1] = p->h2 + 2; box[2] = 1;
    } else if (kind == MK_QUAD_OWN) {
        // [z][y][x][C/4]: a row of RP / 4 floats; the own box is one quad per lane
        dims[0] = (cuuint64_t)g.RP / 4; dims[1] = g.ny; dims[2] = g.nz;
        strides[0] = (cuuint64_t)g.RP; strides[1] = (cuuint64_t)g.PP;   // bytes: RP/4 and PP/4 floats
        box[0] = p->txv; box[1] = p->ty; box[2] = 1;
    } else if (kind == MK_WF_HALO || kind == MK_WF_OWN) {
        if (g.C >= 4) {
            rank = 4;
            dims[0] = g.C; dims[1] = g.nxs; dims[2] = g.ny; dims[3] = g.nz;
            strides[0] = (cuuint64_t)g.C * 4; strides[1] = (cuuint64_t)g.RP * 4;
            strides[2] = (cuuint64_t)g.PP * 4;
            box[0] = g.C; box[1] = cells + (halo ? 2 : 0); box[2] = halo ? rows_h : p->ty; box[3] = 1;
        } else {
            dims[0] = g.RP; dims[1] = g.ny; dims[2] = g.nz;
            strides[0] = (cuuint64_t)g.RP * 4; strides[1] = (cuuint64_t)g.PP * 4;
            box[0] = TXF + (halo ? 8 : 0); box[1] = halo ? rows_h : p->ty; box[2] = 1;
        }
    } else {
        const int es = kind == MK_G_OWN ? 8 : 4;
        if (kind == MK_G_OWN) dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
        dims[0] = g.nxs; dims[1] = g.ny; dims[2] = g.nz;
        strides[0] = (cuuint64_t)g.nxs * es; strides[1] = (cuuint64_t)g.CPP * es;
        box[0] = cells + (kind == MK_CELL_HALO ? 8 : 0);
        box[1] = kind == MK_CELL_HALO ? rows_h : p->ty;
        box[2] = 1;
    }
    for (cuuint32_t d = 0; d < rank; ++d)
        if (box[d] > 256 || box[d] == 0) return set_err(USCT_ERR_ARG, "TMA box dim %u = %u", d, box[d]);
    if ((uintptr_t)ptr % 16 != 0) return set_err(USCT_ERR_ARG, "TMA base address not 16-byte aligned");
    CUtensorMap m;
    CUresult r = enc(&m, dt, rank, const_cast<void*>(ptr), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_err(USCT_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    if (p->maps.size() > 4096) p->maps.clear();
    p->maps.emplace(key, m);
    *out = m;
    return USCT_OK;
}

static int smem_optin() {
    static int v = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    });
    return v;
}

static int check_smem(size_t smem) {
    if (smem > (size_t)smem_optin()) return set_err(USCT_ERR_ARG, "TMA ring needs %zu B of shared memory", smem);
    return USCT_OK;
}

// Opt every TMA kernel into the device's full dynamic shared memory once, at
// plan creation (outside any stream capture).
static void init_tma_attributes() {
    static std::once_flag once;
    std::call_once(once, [] {
        const int b = smem_optin();
        tma_allow_smem<1>(b);  tma_allow_smem<2>(b);  tma_allow_smem<4>(b);
        tma_allow_smem<8>(b);  tma_allow_smem<16>(b); tma_allow_smem<32>(b);
        tma_allow_smem<64>(b);
        cudaGetLastError();
    });
}

// the per-C launchers of usct_tma_inst.cu: 0 = launched, -1 = no kernel
static int tma_fwd_dispatch(int C, const TmaLaunch& t, const FwdArgs& a, const FwdMaps& mp,
                            bool born, bool pcs) {
    switch (C) {
        case 1: return tma_forward<1>(t, a, mp, born, pcs);
        case 2: return tma_forward<2>(t, a, mp, born, pcs);
        case 4: return tma_forward<4>(t, a, mp, born, pcs);
        case 8: return tma_forward<8>(t, a, mp, born, pcs);
        case 16: return tma_forward<16>(t, a, mp, born, pcs);
        case 32: return tma_forward<32>(t, a, mp, born, pcs);
        case 64: return tma_forward<64>(t, a, mp, born, pcs);
        default: return -1;
    }
}
static int tma_adj_dispatch(int C, const TmaLaunch& t, const AdjArgs& a, const AdjMaps& mp) {
    switch (C) {
        case 1: return tma_adjoint<1>(t, a, mp);
        case 2: return tma_adjoint<2>(t, a, mp);
        case 4: return tma_adjoint<4>(t, a, mp);
        case 8: return tma_adjoint<8>(t, a, mp);
        case 16: return tma_adjoint<16>(t, a, mp);
        case 32: return tma_adjoint<32>(t, a, mp);
        case 64: return tma_adjoint<64>(t, a, mp);
        default: return -1;
    }
}

template <bool BORN>
static int launch_fwd_tma(usct_plan* p, const FwdArgs& a0, cudaStream_t s) {
    FwdArgs a = a0;
    a.wait_test = p->wait_test;
    FwdMaps mp;
    memset(&mp, 0, sizeof(mp));
    const bool pcs = p->pcs && !BORN;
    TRY(get_map(p, a.pc, MK_WF_HALO, &mp.pc));
    TRY(get_map(p, a.pp, MK_WF_OWN, &mp.pp));
    TRY(get_map(p, a.S, pcs ? MK_QUAD_OWN : MK_CELL_OWN, &mp.S));
    if (a.sp) TRY(get_map(p, a.sp, MK_CELL_OWN, &mp.sp));
    if (BORN) {
        TRY(get_map(p, a.dc, MK_WF_HALO, &mp.dc));
        TRY(get_map(p, a.dpp, MK_WF_OWN, &mp.dpp));
        TRY(get_map(p, a.vm, MK_CELL_OWN, &mp.vm));
    }
    // per-channel models add a quad row of S to every stage: six 3D stages of
    // the 64x4 / 32-shot tile would no longer let three CTAs share an SM, five do
    const int R = BORN ? p->stages_born
                       : (pcs && p->ndim == 3 ? std::min(p->stages_fwd, 5) : p->stages_fwd);
    const FwdStage L = fwd_stage(p->txv, p->ty, p->ndim == 3, BORN, p->C, p->logC, a.sp != nullptr,
                                 pcs);
    const size_t smem = (size_t)R * L.floats * sizeof(float) + (size_t)R * 8 + 16;
    TRY(check_smem(smem));
    const TmaLaunch t{dim3(p->ntx_t, p->nty_t, p->nzc), smem, R, s, p->d_err, p->txv, p->ty,
                      p->ndim == 3};
    if (tma_fwd_dispatch(p->C, t, a, mp, BORN, pcs) != 0)
        return set_err(USCT_ERR_ARG, "no %dD TMA kernel for tile %dx%d with %d shot channels",
                       p->ndim, p->txv, p->ty, p->C);
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

static int launch_adj_tma(usct_plan* p, const AdjArgs& a0, cudaStream_t s) {
    AdjArgs a = a0;
    a.wait_test = p->wait_test;
    AdjMaps mp;
    memset(&mp, 0, sizeof(mp));
    TRY(get_map(p, a.l1, MK_WF_HALO, &mp.l1));
    TRY(get_map(p, a.S, MK_CELL_HALO, &mp.S));
    TRY(get_map(p, a.l2, MK_WF_OWN, &mp.l2));
    TRY(get_map(p, a.d2, MK_WF_OWN, &mp.d2));
    if (a.sp) TRY(get_map(p, a.sp, MK_CELL_OWN, &mp.sp));
    if (a.gacc) TRY(get_map(p, a.gacc, MK_G_OWN, &mp.g));
    const int R = p->stages_adj;
    const AdjStage L = adj_stage(p->txv, p->ty, p->ndim == 3, p->C, p->logC, a.sp != nullptr,
                                 a.gacc != nullptr);
    const size_t smem = (size_t)R * L.floats * sizeof(float) + (size_t)R * 8 + 16;
    TRY(check_smem(smem));
    const TmaLaunch t{dim3(p->ntx_t, p->nty_t, p->nzc), smem, R, s, p->d_err, p->txv, p->ty,
                      p->ndim == 3};
    if (tma_adj_dispatch(p->C, t, a, mp) != 0)
        return set_err(USCT_ERR_ARG, "no %dD TMA kernel for tile %dx%d with %d shot channels",
                       p->ndim, p->txv, p->ty, p->C);
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

static int tma_fwd2_dispatch(int C, const TmaLaunch2& t, const Fwd2Args& a, const Fwd2Maps& mp) {
    switch (C) {
        case 8: return tma_forward2<8>(t, a, mp);
        case 16: return tma_forward2<16>(t, a, mp);
        case 32: return tma_forward2<32>(t, a, mp);
        case 64: return tma_forward2<64>(t, a, mp);
        default: return -1;
    }
}

// one two-step launch: levels n and n+1 from (p^{n-2}, p^{n-1})
static int launch_fwd2(usct_plan* p, const Fwd2Args& a0, cudaStream_t s) {
    Fwd2Args a = a0;
    a.wait_test = p->wait_test;
    a.g = p->geo;
    a.g.ntiles_x = p->ntx2;
    a.g.zc = p->zc2;
    Fwd2Maps mp;
    memset(&mp, 0, sizeof(mp));
    TRY(get_map(p, a.pc, MK2_A, &mp.A));
    TRY(get_map(p, a.pp, MK2_B, &mp.B));
    TRY(get_map(p, a.S, MK2_S, &mp.S));
    if (a.sp) TRY(get_map(p, a.sp, MK2_S, &mp.sp));
    const size_t smem = tb_smem(p, a.sp != nullptr);
    TRY(check_smem(smem));
    const TmaLaunch2 t{dim3(p->ntx2, p->nty2, p->nzc2), smem, p->ra2, p->rb2, s, p->d_err, p->w2,
                       p->h2};
    if (tma_fwd2_dispatch(p->C, t, a, mp) != 0)
        return set_err(USCT_ERR_ARG, "no two-step kernel for tile %dx%d with %d shot channels",
                       p->w2, p->h2, p->C);
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

template <bool BORN>
static int launch_fwd(usct_plan* p, const FwdArgs& a, cudaStream_t s) {
    if (p->variant == 1) return launch_fwd_tma<BORN>(p, a, s);
    if (p->pcs) return set_err(USCT_ERR_ARG, "per-channel models need the TMA variant");
    const dim3 grid(p->ntx_t, p->nty_t, p->nzc);
    const size_t smem = stencil_smem(p, BORN ? 2 : 1);
    const int key = p->txv * 1000 + p->ty;
    if (p->ndim == 3) {
        switch (key) {
            case 32004: k_forward<32, 4, true, BORN><<<grid, dim3(32, 4), smem, s>>>(a); break;
            case 32008: k_forward<32, 8, true, BORN><<<grid, dim3(32, 8), smem, s>>>(a); break;
            case 64002: k_forward<64, 2, true, BORN><<<grid, dim3(64, 2), smem, s>>>(a); break;
            case 64004: k_forward<64, 4, true, BORN><<<grid, dim3(64, 4), smem, s>>>(a); break;
            default: return set_err(USCT_ERR_ARG, "no 3D kernel for tile %d", key);
        }
    } else {
        switch (key) {
            case 64001: k_forward<64, 1, false, BORN><<<grid, dim3(64, 1), smem, s>>>(a); break;
            case 128001: k_forward<128, 1, false, BORN><<<grid, dim3(128, 1), smem, s>>>(a); break;
            default: return set_err(USCT_ERR_ARG, "no 2D kernel for tile %d", key);
        }
    }
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

static int launch_adj(usct_plan* p, const AdjArgs& a, cudaStream_t s) {
    if (p->variant == 1) return launch_adj_tma(p, a, s);
    const dim3 grid(p->ntx_t, p->nty_t, p->nzc);
    const size_t smem = stencil_smem(p, 1);
    const int key = p->txv * 1000 + p->ty;
    if (p->ndim == 3) {
        switch (key) {
            case 32004: k_adjoint<32, 4, true><<<grid, dim3(32, 4), smem, s>>>(a); break;
            case 32008: k_adjoint<32, 8, true><<<grid, dim3(32, 8), smem, s>>>(a); break;
            case 64002: k_adjoint<64, 2, true><<<grid, dim3(64, 2), smem, s>>>(a); break;
            case 64004: k_adjoint<64, 4, true><<<grid, dim3(64, 4), smem, s>>>(a); break;
            default: return set_err(USCT_ERR_ARG, "no 3D kernel for tile %d", key);
        }
    } else {
        switch (key) {
            case 64001: k_adjoint<64, 1, false><<<grid, dim3(64, 1), smem, s>>>(a); break;
            case 128001: k_adjoint<128, 1, false><<<grid, dim3(128, 1), smem, s>>>(a); break;
            default: return set_err(USCT_ERR_ARG, "no 2D kernel for tile %d", key);
        }
    }
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

// ---- two time levels per forward launch --------------------------------------
// Lay out the two-step tiling (w x h cells per tile) and upload its per-tile
// lists: the sources of each tile grown by one cell and one row (the first
// step computes there), in plane order, and the receivers on each tile's own
// cells in (plane, row, cell) order.
static int tb_configure(usct_plan* p, int w, int h) {
    const Geo& g = p->geo;
    const int C = p->C;
    const int ntx = (g.nxs + w - 1) / w, nty = (g.ny + h - 1) / h, ntiles = ntx * nty;
    int zc = p->zc2_req;
    if (zc <= 0) {
        const long long target = 152LL * 8;   // one CTA per SM: several waves
        long long nzc = (target + ntiles - 1) / ntiles;
        nzc = std::max<long long>(1, std::min<long long>(nzc, g.nz / 8 > 0 ? g.nz / 8 : 1));
        zc = (int)((g.nz + nzc - 1) / nzc);
    }
    zc = std::max(1, std::min(zc, g.nz));
    const int nzc = (g.nz + zc - 1) / zc;
    if (nty > 65535 || nzc > 65535) return set_err(USCT_ERR_ARG, "grid too large for the two-step tiling");
    std::vector<int> sptr((size_t)p->nbatch * (ntiles + 1), 0);
    std::vector<SrcEnt> sent;
    for (int b = 0; b < p->nbatch; ++b) {
        std::vector<std::pair<int, SrcEnt>> tmp;   // (tile, entry)
        for (int c = 0; c < C; ++c) {
            const int t = b * C + c;
            if (t >= p->n_tx) break;
            for (int e = p->h_tx_ptr[t]; e < p->h_tx_ptr[t + 1]; ++e) {
                int z, y, x;
                unravel(p, p->h_tx_cell[e], z, y, x);
                // every tile whose grown region (x0-1 .. x0+w, y0-1 .. y0+h) holds the cell
                for (int yt = std::max(0, (y - h) / h); yt <= std::min(nty - 1, (y + 1) / h); ++yt) {
                    const int ly = y - (yt * h - 1);
                    if (ly < 0 || ly > h + 1) continue;
                    for (int xt = std::max(0, (x - w) / w); xt <= std::min(ntx - 1, (x + 1) / w); ++xt) {
                        const int lx = x - (xt * w - 1);
                        if (lx < 0 || lx > w + 1) continue;
                        tmp.push_back({xt + ntx * yt, SrcEnt{z, ly, lx * C + c, (float)p->h_tx_w[e]}});
                    }
                }
            }
        }
        std::stable_sort(tmp.begin(), tmp.end(), [](const auto& a, const auto& b2) {
            return a.first != b2.first ? a.first < b2.first : a.second.z < b2.second.z;
        });
        int* bp = &sptr[(size_t)b * (ntiles + 1)];
        const int base = (int)sent.size();
        size_t q = 0;
        for (int tl = 0; tl < ntiles; ++tl) {
            bp[tl] = base + (int)q;
            while (q < tmp.size() && tmp[q].first == tl) { sent.push_back(tmp[q].second); ++q; }
        }
        bp[ntiles] = base + (int)q;
    }
    std::vector<std::pair<int, RxEnt>> rtmp;
    for (int j = 0; j < p->n_rx; ++j)
        for (int e = p->h_rx_ptr[j]; e < p->h_rx_ptr[j + 1]; ++e) {
            int z, y, x;
            unravel(p, p->h_rx_cell[e], z, y, x);
            const int xt = x / w, yt = y / h;
            rtmp.push_back({xt + ntx * yt,
                            RxEnt{z, y - yt * h, x - xt * w, e, j, (float)p->h_rx_w[e], 0, 0}});
        }
    std::stable_sort(rtmp.begin(), rtmp.end(), [](const auto& a, const auto& b2) {
        if (a.first != b2.first) return a.first < b2.first;
        if (a.second.z != b2.second.z) return a.second.z < b2.second.z;
        if (a.second.ly != b2.second.ly) return a.second.ly < b2.second.ly;
        return a.second.lcell < b2.second.lcell;
    });
    std::vector<int> rptr(ntiles + 1, 0);
    std::vector<RxEnt> rent;
    {
        size_t q = 0;
        for (int tl = 0; tl < ntiles; ++tl) {
            rptr[tl] = (int)q;
            while (q < rtmp.size() && rtmp[q].first == tl) { rent.push_back(rtmp[q].second); ++q; }
        }
        rptr[ntiles] = (int)q;
    }
    if (sent.empty()) sent.push_back(SrcEnt{0x7fffffff, 0, 0, 0.f});   // never matched
    if (rent.empty()) rent.push_back(RxEnt{0x7fffffff, 0, 0, 0, 0, 0.f, 0, 0});
    free_tb_lists(p);
    int ret;
    if ((ret = upload(&p->d_sptr2, sptr)) != USCT_OK || (ret = upload(&p->d_sent2, sent)) != USCT_OK ||
        (ret = upload(&p->d_rptr2, rptr)) != USCT_OK || (ret = upload(&p->d_rent2, rent)) != USCT_OK) {
        free_tb_lists(p);
        return ret;
    }
    p->w2 = w; p->h2 = h; p->ntx2 = ntx; p->nty2 = nty; p->ntiles2 = ntiles;
    p->zc2 = zc; p->nzc2 = nzc;
    p->maps.clear();   // the two-step boxes changed
    return USCT_OK;
}

extern "C" int usct_plan_set(usct_plan* p, int key, int64_t value) {
    if (!p) return set_err(USCT_ERR_ARG, "null plan");
    switch (key) {
        case USCT_SET_VARIANT:
            if (value != 0 && value != 1) return set_err(USCT_ERR_ARG, "variant must be 0 or 1");
            if (value == 1 && !tma_supported(p))
                return set_err(USCT_ERR_ARG, "the TMA variant needs tile_x*4 >= 4*batch (or tile_x = 32 in 3D)");
            p->variant = (int)value;
            return USCT_OK;
        case USCT_SET_STAGES:
            if (value < 3 || value > 8) return set_err(USCT_ERR_ARG, "stages must be 3..8");
            p->stages_fwd = (int)value;
            p->stages_born = (int)std::max<int64_t>(3, value - 1);
            return USCT_OK;
        case USCT_SET_STAGES_ADJ:
            if (value < 3 || value > 8) return set_err(USCT_ERR_ARG, "stages must be 3..8");
            p->stages_adj = (int)value;
            return USCT_OK;
        case USCT_SET_GRAPHS:
            p->use_graphs = value != 0;
            if (!p->use_graphs) drop_graphs(p);
            return USCT_OK;
        case USCT_SET_WAIT_TEST:
            p->wait_test = value != 0;
            drop_graphs(p);
            return USCT_OK;
        case USCT_SET_TBLOCK: {
            drop_graphs(p);
            if (value == 0) { p->tb = 0; return USCT_OK; }
            // turning it on grows usct_batch_bytes: refuse once workspaces
            // sized without it may be in use
            if (!p->tb && p->launches > 0)
                return set_err(USCT_ERR_STATE, "enable two-step sweeps before the plan's first sweep "
                                               "(it adds two levels to the batch workspace)");
            if (p->ndim != 3 || p->C < 8 || p->variant != 1)
                return set_err(USCT_ERR_ARG, "two-step sweeps need a 3D TMA plan with >= 8 shot channels");
            const int key2 = value == 1 ? tb_default_tile(p->C) : (int)value;
            if (!tb_tile_ok(key2)) return set_err(USCT_ERR_ARG, "unknown two-step tile %d", key2);
            TRY(tb_configure(p, key2 / 100, key2 % 100));
            // shallower rings where the tile's stages do not fit shared memory
            while (tb_smem(p, true) > (size_t)smem_optin() && (p->ra2 > 3 || p->rb2 > 2)) {
                if (p->ra2 > p->rb2 + 1 && p->ra2 > 3) --p->ra2;
                else if (p->rb2 > 2) --p->rb2;
                else --p->ra2;
            }
            if (tb_smem(p, true) > (size_t)smem_optin()) {
                p->tb = 0;
                return set_err(USCT_ERR_ARG, "two-step tile %d needs %zu B of shared memory", key2,
                               tb_smem(p, true));
            }
            p->tb = 1;
            return USCT_OK;
        }
        case USCT_SET_TBLOCK_STAGES: {
            const int ra = (int)(value / 10), rb = (int)(value % 10);
            if (ra < 3 || ra > 6 || rb < 2 || rb > 5)
                return set_err(USCT_ERR_ARG, "two-step stages: 10 * (3..6) + (2..5)");
            const int ra0 = p->ra2, rb0 = p->rb2;
            p->ra2 = ra; p->rb2 = rb;
            if (p->tb && tb_smem(p, true) > (size_t)smem_optin()) {
                p->ra2 = ra0; p->rb2 = rb0;
                return set_err(USCT_ERR_ARG, "two-step rings %d/%d do not fit shared memory", ra, rb);
            }
            drop_graphs(p);
            return USCT_OK;
        }
        case USCT_SET_TBLOCK_ZCHUNK:
            if (value < 0) return set_err(USCT_ERR_ARG, "zchunk must be >= 0");
            p->zc2_req = (int)value;
            drop_graphs(p);
            if (p->w2) return tb_configure(p, p->w2, p->h2);
            return USCT_OK;
        default: return set_err(USCT_ERR_ARG, "unknown setting %d", key);
    }
}

extern "C" int usct_plan_check(usct_plan* p, void* stream) {
    if (!p) return set_err(USCT_ERR_ARG, "null plan");
    CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    int flag = 0;
    CUDA_TRY(cudaMemcpy(&flag, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        CUDA_TRY(cudaMemset(p->d_err, 0, sizeof(int)));
        return set_err(USCT_ERR_CUDA, "a pipelined stencil gave up waiting for its tensor copies");
    }
    return USCT_OK;
}

static int grid1d(long long n, int bs = 256) {
    long long g = (n + bs - 1) / bs;
    return (int)std::max<long long>(1, std::min<long long>(g, 152LL * 32));
}

// ---------------------------------------------------------------------------
// model
// ---------------------------------------------------------------------------
extern "C" int usct_model_prepare(usct_plan* p, void* model_ws, const double* m,
                                  const double* sponge, const double* v, const double* wavelet,
                                  void* stream) {
    Range range_("usct_model_prepare");
    if (!p || !model_ws || !m || !wavelet) return set_err(USCT_ERR_ARG, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    ModelWS M = carve_model(p, model_ws);
    const double dt2 = p->dt * p->dt;
    k_prepare<<<grid1d((long long)p->cells_p), 256, 0, s>>>(m, sponge, v, M.S, M.sp, M.vm, dt2,
                                                           p->geo.nx, p->geo.nxs,
                                                           (long long)p->cells_p);
    k_wavelet<<<(p->nt + 255) / 256, 256, 0, s>>>(wavelet, M.wav, p->nt);
    p->launches += 2;
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemsetAsync(M.g, 0, p->cells_p * sizeof(double), s));
    p->has_sp = sponge != nullptr;
    p->has_vm = v != nullptr;
    return USCT_OK;
}

extern "C" int usct_plan_set_channel_models(usct_plan* p, int n_models, const int* model_of_tx) {
    if (!p || !model_of_tx) return set_err(USCT_ERR_ARG, "null argument");
    if (n_models < 1) return set_err(USCT_ERR_ARG, "need at least one model");
    if (p->launches > 0)
        return set_err(USCT_ERR_STATE, "set per-channel models before the plan's first sweep "
                                       "(they change usct_model_bytes)");
    if (p->variant != 1 || p->C < 4 || p->tb)
        return set_err(USCT_ERR_ARG, "per-channel models need the TMA variant, >= 4 shot channels "
                                     "and one level per launch");
    for (int t = 0; t < p->n_tx; ++t) {
        if (model_of_tx[t] < 0 || model_of_tx[t] >= n_models)
            return set_err(USCT_ERR_ARG, "transmit %d names model %d of %d", t, model_of_tx[t],
                           n_models);
        if (model_of_tx[t] != model_of_tx[t & ~3])
            return set_err(USCT_ERR_ARG, "transmits %d..%d have different models: the model must "
                           "be constant over each group of four transmits", t & ~3, t);
    }
    cudaFree(p->d_tx_model);
    p->d_tx_model = nullptr;
    TRY(upload(&p->d_tx_model, std::vector<int>(model_of_tx, model_of_tx + p->n_tx)));
    p->pcs = 1;
    p->n_models = n_models;
    drop_graphs(p);
    return USCT_OK;
}

extern "C" int usct_model_prepare_channels(usct_plan* p, void* model_ws, const double* models,
                                           const double* wavelet, void* stream) {
    Range range_("usct_model_prepare_channels");
    if (!p || !model_ws || !models || !wavelet) return set_err(USCT_ERR_ARG, "null argument");
    if (!p->pcs) return set_err(USCT_ERR_STATE, "the plan has no per-channel models");
    cudaStream_t s = (cudaStream_t)stream;
    ModelWS M = carve_model(p, model_ws);
    const size_t spf = spc_floats(p);
    // batch b's S starts at b * spf
    for (int b = 0; b < p->nbatch; ++b) {
        k_prepare_channels<<<grid1d((long long)p->LV / 4), 256, 0, s>>>(
            models, p->d_tx_model + (size_t)b * p->C, M.Spc + (size_t)b * spf, p->dt * p->dt,
            p->geo.nx, p->geo.nxs, p->C, p->logC, std::min(p->C, p->n_tx - b * p->C),
            (long long)p->cells_p, (long long)p->LV / 4);
        ++p->launches;
    }
    k_wavelet<<<(p->nt + 255) / 256, 256, 0, s>>>(wavelet, M.wav, p->nt);
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    p->has_sp = false;
    p->has_vm = false;
    return USCT_OK;
}

extern "C" int usct_model_gradient(usct_plan* p, void* model_ws, const double* m, double* grad,
                                   void* stream) {
    Range range_("usct_model_gradient");
    if (!p || !model_ws || !m || !grad) return set_err(USCT_ERR_ARG, "null argument");
    ModelWS M = carve_model(p, model_ws);
    k_finalize<<<grid1d((long long)p->cells_p), 256, 0, (cudaStream_t)stream>>>(
        M.g, m, grad, p->geo.nx, p->geo.nxs, (long long)p->cells_p);
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

// ---------------------------------------------------------------------------
// batch sweeps
// ---------------------------------------------------------------------------
static int gather(usct_plan* p, const BatchWS& B, int b, float* out, const float* dobs, int mode,
                  cudaStream_t s, const float* tw = nullptr) {
    const int shot0 = b * p->C;
    const int nb = std::min(p->C, p->n_tx - shot0);
    k_gather<<<JBLK, 256, 0, s>>>(B.rs, p->nslot, p->C, p->logC, p->nt, p->n_rx, p->d_rxptr, shot0,
                                  nb, out, dobs, B.res, mode, B.jpart, tw);
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

// Run `enqueue` directly, or -- with graphs on and a capturable stream -- as a
// CUDA graph captured on first use for this (op, batch, mode, buffers) key and
// replayed afterwards (the kernels read everything else from the buffers, so
// a replay recomputes with the buffers' current contents).
static int run_graph(usct_plan* p, cudaStream_t s, int op, int b, int mode, const void* k0,
                     const void* k1, const void* k2, const std::function<int()>& enqueue) {
    if (!p->use_graphs || s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread)
        return enqueue();
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    CUDA_TRY(cudaStreamIsCapturing(s, &st));
    if (st != cudaStreamCaptureStatusNone) return enqueue();   // the caller is capturing
    const auto key = std::make_tuple(op, b, mode, k0, k1, k2);
    auto it = p->graphs.find(key);
    if (it == p->graphs.end()) {
        if (p->graphs.size() >= 64) drop_graphs(p);
        const long long before = p->launches;
        CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue();
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (rc != USCT_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        CUDA_TRY(e);
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        CUDA_TRY(ei);
        it = p->graphs.emplace(key, usct_plan::Captured{exec, p->launches - before}).first;
        p->launches = before;
    }
    CUDA_TRY(cudaGraphLaunch(it->second.exec, s));
    p->launches += it->second.kernels;
    return USCT_OK;
}

static int batch_forward_impl(usct_plan* p, const void* model_ws, void* batch_ws, int b, int mode,
                              float* traces, cudaStream_t s);

extern "C" int usct_batch_forward(usct_plan* p, const void* model_ws, void* batch_ws, int b,
                                  int mode, float* traces, void* stream) {
    Range range_("usct_batch_forward");
    if (!p || !model_ws || !batch_ws) return set_err(USCT_ERR_ARG, "null argument");
    if (b < 0 || b >= p->nbatch) return set_err(USCT_ERR_ARG, "batch %d out of range", b);
    if (mode < USCT_MODE_FORWARD || mode > USCT_MODE_BORN) return set_err(USCT_ERR_ARG, "bad mode");
    if (mode == USCT_MODE_BORN && !p->has_vm)
        return set_err(USCT_ERR_STATE, "Born sweep needs a model prepared with v");
    if (p->pcs && mode != USCT_MODE_FORWARD)
        return set_err(USCT_ERR_ARG, "a plan with per-channel models runs forward sweeps only");
    cudaStream_t s = (cudaStream_t)stream;
    // the sponge choice is baked into captured launches: key on it too
    const void* k2 = (const void*)((uintptr_t)traces ^ (p->has_sp ? (uintptr_t)1 : 0));
    return run_graph(p, s, 1, b, mode, model_ws, batch_ws, k2,
                     [&] { return batch_forward_impl(p, model_ws, batch_ws, b, mode, traces, s); });
}

// The checkpoint copy and the stash slot of level n in a gradient's forward
// sweep: the pair (p^{a-1}, p^a) at every segment start a = j*k, and the d2p
// of the last segment's levels.
static void level_outputs(const usct_plan* p, const BatchWS& B, int mode, int n, float*& ck,
                          float*& d2) {
    ck = nullptr;
    d2 = nullptr;
    if (mode < USCT_MODE_GRADIENT) return;
    const size_t lvf = al256(p->LV * sizeof(float)) / sizeof(float);
    const int k = p->k, nt = p->nt, al = (p->nseg - 1) * k;
    if ((n + 1) % k == 0 && n + 1 < nt - 1) ck = B.ck + (size_t)((n + 1) / k) * 2 * lvf;
    else if (n % k == 0 && n < nt - 1) ck = B.ck + ((size_t)(n / k) * 2 + 1) * lvf;
    if (n > al) d2 = B.stash + (size_t)(n - al - 1) * lvf;
}

// Forward sweep with two levels per launch: state pairs (p^{n-2}, p^{n-1}) in
// {P[0], P[1]} and {P2[0], P2[1]} alternately (the two-step kernel reads both
// inputs with halos, so it never writes in place); an odd last level takes one
// single-step launch.
static int forward_sweep_tb(usct_plan* p, const ModelWS& M, const BatchWS& B, int b, int mode,
                            cudaStream_t s) {
    float* st[4] = {B.P[0], B.P[1], B.P2[0], B.P2[1]};
    int prev = 0, cur = 1;   // p^{n-2}, p^{n-1} (both zero at n = 1)
    const int nt = p->nt;
    const size_t row = (size_t)p->nslot * p->C;
    for (int n = 1; n < nt;) {
        if (n + 1 <= nt - 1) {
            const int o = prev >= 2 ? 0 : 2;
            Fwd2Args a{};
            a.pc = st[cur];
            a.pp = st[prev];
            a.pn1 = st[o];
            a.pn2 = st[o + 1];
            a.S = M.S;
            a.sp = p->has_sp ? M.sp : nullptr;
            a.wav = M.wav;
            a.n = n;
            level_outputs(p, B, mode, n, a.ck1, a.d21);
            level_outputs(p, B, mode, n + 1, a.ck2, a.d22);
            a.s_ptr = p->d_sptr2 + (size_t)b * (p->ntiles2 + 1);
            a.s_ent = p->d_sent2;
            a.r_ptr = p->d_rptr2;
            a.r_ent = p->d_rent2;
            a.rs1 = B.rs + (size_t)n * row;
            a.rs2 = B.rs + (size_t)(n + 1) * row;
            TRY(launch_fwd2(p, a, s));
            prev = o;
            cur = o + 1;
            n += 2;
        } else {
            FwdArgs a{};
            a.g = p->geo;
            a.pc = st[cur];
            a.pp = st[prev];
            a.pn = st[prev];
            a.S = M.S;
            a.sp = p->has_sp ? M.sp : nullptr;
            a.wav = M.wav;
            a.n = n;
            level_outputs(p, B, mode, n, a.ck, a.d2);
            a.s_ptr = p->d_sptr + (size_t)b * (p->ntiles + 1);
            a.s_ent = p->d_sent;
            a.r_ptr = p->d_rptr;
            a.r_ent = p->d_rent;
            a.rs = B.rs + (size_t)n * row;
            TRY(launch_fwd<false>(p, a, s));
            n += 1;
        }
    }
    return USCT_OK;
}

static int batch_forward_impl(usct_plan* p, const void* model_ws, void* batch_ws, int b, int mode,
                              float* traces, cudaStream_t s) {
    const ModelWS M = carve_model(p, (void*)model_ws);
    const BatchWS B = carve_batch(p, batch_ws, mode);
    const size_t lvb = al256(p->LV * sizeof(float));
    CUDA_TRY(cudaMemsetAsync(B.P[0], 0, 2 * lvb, s));
    CUDA_TRY(cudaMemsetAsync(B.rs, 0, (size_t)p->nslot * p->C * sizeof(float), s));
    if (mode == USCT_MODE_BORN) CUDA_TRY(cudaMemsetAsync(B.D[0], 0, 2 * lvb, s));
    if (mode >= USCT_MODE_GRADIENT) CUDA_TRY(cudaMemsetAsync(B.ck, 0, 2 * lvb, s));
    if (tb_on(p) && mode != USCT_MODE_BORN) {
        TRY(forward_sweep_tb(p, M, B, b, mode, s));
        return gather(p, B, b, traces, nullptr, 0, s);
    }
    const size_t lvf = lvb / sizeof(float);
    const float* Sb = p->pcs ? M.Spc + (size_t)b * spc_floats(p) : M.S;   // this batch's S
    const int k = p->k, nt = p->nt;
    const int al = (p->nseg - 1) * k;
    for (int n = 1; n < nt; ++n) {
        FwdArgs a{};
        a.g = p->geo;
        a.pc = B.P[(n - 1) & 1];
        a.pp = B.P[n & 1];
        a.pn = B.P[n & 1];
        a.S = Sb;
        a.sp = p->has_sp ? M.sp : nullptr;
        a.wav = M.wav;
        a.n = n;
        if (mode >= USCT_MODE_GRADIENT) {
            if ((n + 1) % k == 0 && n + 1 < nt - 1) a.ck = B.ck + (size_t)((n + 1) / k) * 2 * lvf;
            else if (n % k == 0 && n < nt - 1) a.ck = B.ck + ((size_t)(n / k) * 2 + 1) * lvf;
            if (n > al) a.d2 = B.stash + (size_t)(n - al - 1) * lvf;
        }
        a.s_ptr = p->d_sptr + (size_t)b * (p->ntiles + 1);
        a.s_ent = p->d_sent;
        a.r_ptr = p->d_rptr;
        a.r_ent = p->d_rent;
        a.rs = B.rs + (size_t)n * p->nslot * p->C;
        if (mode == USCT_MODE_BORN) {
            a.dc = B.D[(n - 1) & 1];
            a.dpp = B.D[n & 1];
            a.dn = B.D[n & 1];
            a.vm = M.vm;
            TRY(launch_fwd<true>(p, a, s));
        } else {
            TRY(launch_fwd<false>(p, a, s));
        }
    }
    return gather(p, B, b, traces, nullptr, mode == USCT_MODE_BORN ? 2 : 0, s);
}

extern "C" int usct_batch_misfit(usct_plan* p, void* batch_ws, int b, const float* dobs, double* J,
                                 void* stream) {
    return usct_batch_misfit_tw(p, batch_ws, b, dobs, nullptr, 0, J, stream);
}

extern "C" int usct_batch_misfit_mt(usct_plan* p, void* batch_ws, int b, const float* dobs,
                                    int misfit_type, double* J, void* stream) {
    return usct_batch_misfit_tw(p, batch_ws, b, dobs, nullptr, misfit_type, J, stream);
}

static int batch_misfit_l2(usct_plan* p, void* batch_ws, int b, const float* dobs,
                           const float* tw, double* J, cudaStream_t s) {
    const BatchWS B = carve_batch(p, batch_ws, USCT_MODE_FORWARD);
    TRY(gather(p, B, b, nullptr, dobs, 1, s, tw));
    if (J) {
        const int shot0 = b * p->C;
        const int nb = std::min(p->C, p->n_tx - shot0);
        k_jsum<<<1, 64, 0, s>>>(B.jpart, p->C, JBLK, shot0, nb, J);
        ++p->launches;
        CUDA_TRY(cudaGetLastError());
    }
    return USCT_OK;
}

extern "C" int usct_batch_misfit_tw(usct_plan* p, void* batch_ws, int b, const float* dobs,
                                    const float* weights, int misfit_type, double* J,
                                    void* stream) {
    Range range_("usct_batch_misfit_tw");
    if (!p || !batch_ws || !dobs) return set_err(USCT_ERR_ARG, "null argument");
    if (misfit_type != 0 && misfit_type != 1)
        return set_err(USCT_ERR_ARG, "misfit_type must be 0 (L2) or 1 (GCN)");
    if (b < 0 || b >= p->nbatch) return set_err(USCT_ERR_ARG, "batch %d out of range", b);
    cudaStream_t s = (cudaStream_t)stream;
    if (misfit_type == 0) return batch_misfit_l2(p, batch_ws, b, dobs, weights, J, s);
    const BatchWS B = carve_batch(p, batch_ws, USCT_MODE_FORWARD);
    TRY(gather(p, B, b, nullptr, nullptr, 2, s, weights));   // res = (windowed) traces
    const int shot0 = b * p->C;
    const int nb = std::min(p->C, p->n_tx - shot0);
    const int n = p->n_rx * p->C;
    k_gcn<<<(n + 31) / 32, dim3(32, kGS), 0, s>>>(B.res, dobs, p->C, p->logC, p->nt, p->n_rx, shot0,
                                                  nb, B.gj, weights);
    ++p->launches;
    if (J) {
        k_gcn_j<<<1, 64, 0, s>>>(B.gj, p->C, p->n_rx, shot0, nb, J);
        ++p->launches;
    }
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

extern "C" int usct_batch_adjoint_source(usct_plan* p, void* batch_ws, int b, const float* adj,
                                         void* stream) {
    if (!p || !batch_ws || !adj) return set_err(USCT_ERR_ARG, "null argument");
    if (b < 0 || b >= p->nbatch) return set_err(USCT_ERR_ARG, "batch %d out of range", b);
    const BatchWS B = carve_batch(p, batch_ws, USCT_MODE_FORWARD);
    const int shot0 = b * p->C;
    const int nb = std::min(p->C, p->n_tx - shot0);
    k_adjsrc<<<grid1d((long long)p->nt * p->n_rx * p->C), 256, 0, (cudaStream_t)stream>>>(
        adj, B.res, p->C, p->nt, p->n_rx, shot0, nb);
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

static int batch_backward_impl(usct_plan* p, void* model_ws, void* batch_ws, int b, cudaStream_t s);

extern "C" int usct_batch_backward(usct_plan* p, void* model_ws, void* batch_ws, int b, void* stream) {
    Range range_("usct_batch_backward");
    if (!p || !model_ws || !batch_ws) return set_err(USCT_ERR_ARG, "null argument");
    if (b < 0 || b >= p->nbatch) return set_err(USCT_ERR_ARG, "batch %d out of range", b);
    cudaStream_t s = (cudaStream_t)stream;
    const void* k2 = (const void*)(uintptr_t)(p->has_sp ? 1 : 0);
    return run_graph(p, s, 2, b, 0, model_ws, batch_ws, k2,
                     [&] { return batch_backward_impl(p, model_ws, batch_ws, b, s); });
}

static int batch_backward_impl(usct_plan* p, void* model_ws, void* batch_ws, int b, cudaStream_t s) {
    const ModelWS M = carve_model(p, model_ws);
    const BatchWS B = carve_batch(p, batch_ws, USCT_MODE_GRADIENT);
    const size_t lvb = al256(p->LV * sizeof(float));
    const size_t lvf = lvb / sizeof(float);
    CUDA_TRY(cudaMemsetAsync(B.L[0], 0, 2 * lvb, s));
    const int k = p->k, nt = p->nt;
    float* W[2] = {B.P[0], B.P[1]};
    for (int j = p->nseg - 1; j >= 0; --j) {
        const int a0 = j * k;
        const int b1 = std::min(a0 + k, nt - 1);
        const float* ck0 = B.ck + (size_t)j * 2 * lvf;
        const float* ck1 = ck0 + lvf;
        if (j != p->nseg - 1 && tb_on(p)) {
            // the segment's levels two at a time from the stored pair, into
            // the state pairs {P[0], P[1]} and {P2[0], P2[1]} alternately
            float* pair[2][2] = {{B.P[0], B.P[1]}, {B.P2[0], B.P2[1]}};
            const float* prevp = ck0;
            const float* curp = ck1;
            int out = 0;
            for (int n = a0 + 1; n <= b1;) {
                if (n + 1 <= b1) {
                    Fwd2Args a{};
                    a.pc = curp;
                    a.pp = prevp;
                    a.pn1 = pair[out][0];
                    a.pn2 = pair[out][1];
                    a.S = M.S;
                    a.sp = p->has_sp ? M.sp : nullptr;
                    a.wav = M.wav;
                    a.n = n;
                    a.d21 = B.stash + (size_t)(n - a0 - 1) * lvf;
                    a.d22 = B.stash + (size_t)(n - a0) * lvf;
                    a.s_ptr = p->d_sptr2 + (size_t)b * (p->ntiles2 + 1);
                    a.s_ent = p->d_sent2;
                    a.r_ptr = p->d_rptr2;
                    a.r_ent = p->d_rent2;
                    TRY(launch_fwd2(p, a, s));
                    prevp = pair[out][0];
                    curp = pair[out][1];
                    out ^= 1;
                    n += 2;
                } else {
                    FwdArgs a{};
                    a.g = p->geo;
                    a.pc = curp;
                    a.pp = prevp;
                    // in place over p^{n-2}, unless that is the stored checkpoint
                    a.pn = prevp == ck0 ? pair[out][0] : const_cast<float*>(prevp);
                    a.S = M.S;
                    a.sp = p->has_sp ? M.sp : nullptr;
                    a.wav = M.wav;
                    a.n = n;
                    a.d2 = B.stash + (size_t)(n - a0 - 1) * lvf;
                    a.s_ptr = p->d_sptr + (size_t)b * (p->ntiles + 1);
                    a.s_ent = p->d_sent;
                    a.r_ptr = p->d_rptr;
                    a.r_ent = p->d_rent;
                    TRY(launch_fwd<false>(p, a, s));
                    n += 1;
                }
            }
        } else if (j != p->nseg - 1) {
            for (int n = a0 + 1; n <= b1; ++n) {
                FwdArgs a{};
                a.g = p->geo;
                a.pc = (n == a0 + 1) ? ck1 : W[(n - 1) & 1];
                a.pp = (n == a0 + 1) ? ck0 : (n == a0 + 2 ? ck1 : W[n & 1]);
                a.pn = W[n & 1];
                a.S = M.S;
                a.sp = p->has_sp ? M.sp : nullptr;
                a.wav = M.wav;
                a.n = n;
                a.d2 = B.stash + (size_t)(n - a0 - 1) * lvf;
                a.s_ptr = p->d_sptr + (size_t)b * (p->ntiles + 1);
                a.s_ent = p->d_sent;
                a.r_ptr = p->d_rptr;
                a.r_ent = p->d_rent;
                TRY(launch_fwd<false>(p, a, s));
            }
        }
        for (int kk = b1; kk >= a0 + 1; --kk) {
            AdjArgs a{};
            a.g = p->geo;
            a.l1 = B.L[(kk + 1) & 1];
            a.l2 = B.L[kk & 1];
            a.lk = B.L[kk & 1];
            a.S = M.S;
            a.sp = p->has_sp ? M.sp : nullptr;
            a.d2 = B.stash + (size_t)(kk - a0 - 1) * lvf;
            a.gacc = M.g;
            a.r_ptr = p->d_rptr;
            a.r_ent = p->d_rent;
            a.res = B.res + (size_t)kk * p->n_rx * p->C;
            TRY(launch_adj(p, a, s));
        }
    }
    return USCT_OK;
}

// ---------------------------------------------------------------------------
// whole-acquisition device calls
// ---------------------------------------------------------------------------
extern "C" int usct_forward_fmc_dev(usct_plan* p, const double* m, const double* sponge,
                                    const double* wavelet, float* data, void* model_ws,
                                    void* batch_ws, void* stream) {
    Range range_("usct_forward_fmc_dev");
    TRY(usct_model_prepare(p, model_ws, m, sponge, nullptr, wavelet, stream));
    for (int b = 0; b < p->nbatch; ++b)
        TRY(usct_batch_forward(p, model_ws, batch_ws, b, USCT_MODE_FORWARD, data, stream));
    return USCT_OK;
}

extern "C" int usct_misfit_and_gradient_dev(usct_plan* p, const double* m, const double* sponge,
                                            const double* wavelet, const float* dobs, double* J,
                                            double* grad, void* model_ws, void* batch_ws,
                                            void* stream) {
    TRY(usct_model_prepare(p, model_ws, m, sponge, nullptr, wavelet, stream));
    for (int b = 0; b < p->nbatch; ++b) {
        TRY(usct_batch_forward(p, model_ws, batch_ws, b, USCT_MODE_GRADIENT, nullptr, stream));
        TRY(usct_batch_misfit(p, batch_ws, b, dobs, J, stream));
        TRY(usct_batch_backward(p, model_ws, batch_ws, b, stream));
    }
    return usct_model_gradient(p, model_ws, m, grad, stream);
}

extern "C" int usct_misfit_and_gradient_mt_dev(usct_plan* p, const double* m, const double* sponge,
                                               const double* wavelet, const float* dobs,
                                               int misfit_type, double* J, double* grad,
                                               void* model_ws, void* batch_ws, void* stream) {
    return usct_misfit_and_gradient_tw_dev(p, m, sponge, wavelet, dobs, nullptr, misfit_type, J,
                                           grad, model_ws, batch_ws, stream);
}

extern "C" int usct_misfit_and_gradient_tw_dev(usct_plan* p, const double* m, const double* sponge,
                                               const double* wavelet, const float* dobs,
                                               const float* weights, int misfit_type, double* J,
                                               double* grad, void* model_ws, void* batch_ws,
                                               void* stream) {
    Range range_("usct_misfit_and_gradient_tw_dev");
    if (misfit_type != 0 && misfit_type != 1)
        return set_err(USCT_ERR_ARG, "misfit_type must be 0 (L2) or 1 (GCN)");
    TRY(usct_model_prepare(p, model_ws, m, sponge, nullptr, wavelet, stream));
    for (int b = 0; b < p->nbatch; ++b) {
        TRY(usct_batch_forward(p, model_ws, batch_ws, b, USCT_MODE_GRADIENT, nullptr, stream));
        TRY(usct_batch_misfit_tw(p, batch_ws, b, dobs, weights, misfit_type, J, stream));
        TRY(usct_batch_backward(p, model_ws, batch_ws, b, stream));
    }
    return usct_model_gradient(p, model_ws, m, grad, stream);
}

extern "C" int usct_gn_hessian_vector_dev(usct_plan* p, const double* m, const double* sponge,
                                          const double* wavelet, const double* v, double* hv,
                                          float* born, void* model_ws, void* batch_ws,
                                          void* stream) {
    Range range_("usct_gn_hessian_vector_dev");
    if (!v) return set_err(USCT_ERR_ARG, "v is null");
    TRY(usct_model_prepare(p, model_ws, m, sponge, v, wavelet, stream));
    for (int b = 0; b < p->nbatch; ++b) {
        TRY(usct_batch_forward(p, model_ws, batch_ws, b, USCT_MODE_BORN, born, stream));
        TRY(usct_batch_backward(p, model_ws, batch_ws, b, stream));
    }
    return usct_model_gradient(p, model_ws, m, hv, stream);
}

// ---------------------------------------------------------------------------
// host-pointer calls with the reference core's signatures
// ---------------------------------------------------------------------------
namespace {
struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};
}  // namespace

static int host_plan(usct_plan** plan, const int* dims, int ndim, double h, double dt, int nt,
                     const int* tx_lin, int n_tx, const int* rec_lin, int n_rec) {
    if (!tx_lin || !rec_lin) return set_err(USCT_ERR_ARG, "null index array");
    std::vector<int> tp(n_tx + 1), rp(n_rec + 1);
    std::vector<int64_t> tc(n_tx), rc(n_rec);
    std::vector<double> tw(n_tx, 1.0), rw(n_rec, 1.0);
    for (int i = 0; i <= n_tx; ++i) tp[i] = i;
    for (int i = 0; i <= n_rec; ++i) rp[i] = i;
    for (int i = 0; i < n_tx; ++i) tc[i] = tx_lin[i];
    for (int i = 0; i < n_rec; ++i) rc[i] = rec_lin[i];
    return usct_plan_create(plan, ndim, dims, h, dt, nt, n_tx, tp.data(), tc.data(), tw.data(), n_rec,
                            rp.data(), rc.data(), rw.data(), 0, 0, 0, 0, 0);
}

extern "C" int usct_forward_fmc(const double* m, const int* dims, int ndim, double h, double dt, int nt,
                                const int* tx_lin, int n_tx, const int* rec_lin, int n_rec,
                                const double* wavelet, double* data) {
    if (!m || !wavelet || !data) return set_err(USCT_ERR_ARG, "null argument");
    usct_plan* p = nullptr;
    TRY(host_plan(&p, dims, ndim, h, dt, nt, tx_lin, n_tx, rec_lin, n_rec));
    struct Guard { usct_plan* p; ~Guard() { usct_plan_destroy(p); } } guard{p};
    const size_t nd = (size_t)n_tx * nt * n_rec;
    DevBuf dm, dw, dd, mws, bws;
    CUDA_TRY(cudaMalloc(&dm.p, p->N * sizeof(double)));
    CUDA_TRY(cudaMalloc(&dw.p, (size_t)nt * sizeof(double)));
    CUDA_TRY(cudaMalloc(&dd.p, nd * sizeof(float)));
    CUDA_TRY(cudaMalloc(&mws.p, usct_model_bytes(p)));
    CUDA_TRY(cudaMalloc(&bws.p, usct_batch_bytes(p, USCT_MODE_FORWARD)));
    CUDA_TRY(cudaMemcpy(dm.p, m, p->N * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dw.p, wavelet, (size_t)nt * sizeof(double), cudaMemcpyHostToDevice));
    TRY(usct_forward_fmc_dev(p, (const double*)dm.p, nullptr, (const double*)dw.p, (float*)dd.p,
                             mws.p, bws.p, nullptr));
    std::vector<float> hf(nd);
    CUDA_TRY(cudaMemcpy(hf.data(), dd.p, nd * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < nd; ++i) data[i] = hf[i];
    return USCT_OK;
}

extern "C" int usct_misfit_and_gradient_mt(const double* m, const int* dims, int ndim, double h,
                                           double dt, int nt, const int* tx_lin, int n_tx,
                                           const int* rec_lin, int n_rec, const double* wavelet,
                                           const double* dobs, double* grad, int misfit_type,
                                           double* J);

extern "C" int usct_misfit_and_gradient(const double* m, const int* dims, int ndim, double h,
                                        double dt, int nt, const int* tx_lin, int n_tx,
                                        const int* rec_lin, int n_rec, const double* wavelet,
                                        const double* dobs, double* grad, double* J) {
    return usct_misfit_and_gradient_mt(m, dims, ndim, h, dt, nt, tx_lin, n_tx, rec_lin, n_rec,
                                       wavelet, dobs, grad, 0, J);
}

extern "C" int usct_misfit_and_gradient_mt(const double* m, const int* dims, int ndim, double h,
                                           double dt, int nt, const int* tx_lin, int n_tx,
                                           const int* rec_lin, int n_rec, const double* wavelet,
                                           const double* dobs, double* grad, int misfit_type,
                                           double* J) {
    if (!m || !wavelet || !dobs || !grad) return set_err(USCT_ERR_ARG, "null argument");
    usct_plan* p = nullptr;
    TRY(host_plan(&p, dims, ndim, h, dt, nt, tx_lin, n_tx, rec_lin, n_rec));
    struct Guard { usct_plan* p; ~Guard() { usct_plan_destroy(p); } } guard{p};
    const size_t nd = (size_t)n_tx * nt * n_rec;
    std::vector<float> hdobs(nd);
    for (size_t i = 0; i < nd; ++i) hdobs[i] = (float)dobs[i];
    DevBuf dm, dw, dob, dJ, dg, mws, bws;
    CUDA_TRY(cudaMalloc(&dm.p, p->N * sizeof(double)));
    CUDA_TRY(cudaMalloc(&dw.p, (size_t)nt * sizeof(double)));
    CUDA_TRY(cudaMalloc(&dob.p, nd * sizeof(float)));
    CUDA_TRY(cudaMalloc(&dJ.p, (size_t)n_tx * sizeof(double)));
    CUDA_TRY(cudaMalloc(&dg.p, p->N * sizeof(double)));
    CUDA_TRY(cudaMalloc(&mws.p, usct_model_bytes(p)));
    CUDA_TRY(cudaMalloc(&bws.p, usct_batch_bytes(p, USCT_MODE_GRADIENT)));
    CUDA_TRY(cudaMemcpy(dm.p, m, p->N * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dw.p, wavelet, (size_t)nt * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dob.p, hdobs.data(), nd * sizeof(float), cudaMemcpyHostToDevice));
    TRY(usct_misfit_and_gradient_mt_dev(p, (const double*)dm.p, nullptr, (const double*)dw.p,
                                        (const float*)dob.p, misfit_type, (double*)dJ.p,
                                        (double*)dg.p, mws.p, bws.p, nullptr));
    std::vector<double> hJ(n_tx);
    CUDA_TRY(cudaMemcpy(hJ.data(), dJ.p, (size_t)n_tx * sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(grad, dg.p, p->N * sizeof(double), cudaMemcpyDeviceToHost));
    if (J) {
        double s = 0.0;
        for (int t = 0; t < n_tx; ++t) s += hJ[t];
        *J = s;
    }
    return USCT_OK;
}

// The plain one-shot-per-launch form needs the plan internals declared above.
#include "usct_plain.cuh"
