// Library-wide C ABI pieces: error reporting, version, per-kernel timing.
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include "common.cuh"

namespace matpl {
namespace {
thread_local std::string g_last_error;
std::mutex g_prof_mu;
bool g_prof_on = false;
std::vector<cudaEvent_t> g_pool;
size_t g_pool_next = 0;
struct Rec {
    std::string name;
    cudaEvent_t a, b;
};
std::vector<Rec> g_recs;
}  // namespace

void set_error(const std::string &msg) { g_last_error = msg; }

int device_sms() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        dev = 0;
    }
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return 148;                    // a Blackwell-class part; only sizes grids
    }
    cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

int require_current_device(const void *p, const char *what) {
    if (p == nullptr) return MATPL_OK;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();            // not a pointer the runtime knows: nothing to compare
        return MATPL_OK;
    }
    if (a.type != cudaMemoryTypeDevice) return MATPL_OK;
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) {
        set_error(std::string(what) + ": no current CUDA device");
        return MATPL_ERR_CUDA;
    }
    if (a.device != cur) {
        set_error(std::string(what) + ": arrays live on GPU " + std::to_string(a.device) +
                  " but GPU " + std::to_string(cur) +
                  " is current; make the arrays' device current before the call");
        return MATPL_ERR_INVALID;
    }
    return MATPL_OK;
}

bool profiling_enabled() { return g_prof_on; }

cudaEvent_t profile_event() {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (g_pool_next >= g_pool.size()) return nullptr;
    return g_pool[g_pool_next++];
}

void profile_record(const char *name, cudaEvent_t a, cudaEvent_t b) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_recs.push_back({name, a, b});
}
}  // namespace matpl

using namespace matpl;

extern "C" const char *matpl_last_error(void) { return g_last_error.c_str(); }
extern "C" int matpl_version(void) { return 1; }

extern "C" int matpl_profile_begin(int max_launches) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    MATPL_REQUIRE(max_launches > 0 && max_launches <= (1 << 20), MATPL_ERR_INVALID,
                  "max_launches out of range");
    const size_t need = 2 * (size_t)max_launches;
    while (g_pool.size() < need) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) {
            set_error("matpl_profile_begin: cudaEventCreate failed");
            return MATPL_ERR_CUDA;
        }
        g_pool.push_back(e);
    }
    g_pool_next = 0;
    g_recs.clear();
    g_prof_on = true;
    return MATPL_OK;
}

extern "C" int matpl_profile_collect(int max_names, char *names, int name_len, double *total_ms,
                                     int *launches, int *n_out) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    MATPL_REQUIRE(n_out && (max_names <= 0 || (names && name_len > 0 && total_ms && launches)),
                  MATPL_ERR_INVALID, "matpl_profile_collect: null output array or name_len <= 0");
    g_prof_on = false;
    std::map<std::string, std::pair<double, int>> agg;
    for (auto &r : g_recs) {
        if (cudaEventSynchronize(r.b) != cudaSuccess) {
            set_error("matpl_profile_collect: cudaEventSynchronize failed");
            return MATPL_ERR_CUDA;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        auto &x = agg[r.name];
        x.first += ms;
        x.second += 1;
    }
    int k = 0;
    for (auto &kv : agg) {
        if (k >= max_names) break;
        snprintf(names + (size_t)k * name_len, name_len, "%s", kv.first.c_str());
        total_ms[k] = kv.second.first;
        launches[k] = kv.second.second;
        ++k;
    }
    *n_out = k;
    g_recs.clear();
    g_pool_next = 0;
    return MATPL_OK;
}
