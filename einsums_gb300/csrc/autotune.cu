// Tile autotuner cache: per shape bucket, the choice measured on this device,
// persisted as "key=value" lines keyed by GPU name, SM count and library
// version so a cache from another GPU or build is never reused.
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <sys/stat.h>

#include "grouped.cuh"

namespace eg::autotune {

namespace {
std::mutex &g_mu = *new std::mutex;
bool g_loaded = false;
std::map<std::string, int> &g_cache = *new std::map<std::string, int>;

int ceil_log2(int64_t x) {
    int l = 0;
    while ((int64_t(1) << l) < x) l++;
    return l;
}

std::string device_tag() {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, dev);
    std::ostringstream o;
    o << prop.name << "/sm" << prop.major << prop.minor << "/" << prop.multiProcessorCount << "/" << eg_version();
    return o.str();
}

void load_locked() {
    if (g_loaded) return;
    g_loaded = true;
    std::ifstream f(cache_path());
    std::string line;
    while (std::getline(f, line)) {
        const auto eq = line.rfind('=');
        if (eq == std::string::npos) continue;
        g_cache[line.substr(0, eq)] = std::atoi(line.c_str() + eq + 1);
    }
}

void mkdirs(const std::string &path) {
    for (size_t i = 1; i < path.size(); i++)
        if (path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
}
} // namespace

std::string cache_path() {
    if (const char *p = std::getenv("EINSUMS_GB300_AUTOTUNE_CACHE")) return p;
    const char *home = std::getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/einsums_gb300/autotune.txt";
}

bool enabled() {
    const char *v = std::getenv("EINSUMS_GB300_AUTOTUNE");
    return !(v && std::string(v) == "0");
}

std::string bucket_key(const char *mode, int64_t M, int64_t N, int64_t K) {
    std::ostringstream o;
    o << mode << "|" << ceil_log2(M) << "|" << ceil_log2(N) << "|" << ceil_log2(K);
    return o.str();
}

bool lookup(const std::string &bucket, int *choice) {
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    auto it = g_cache.find(device_tag() + "|" + bucket);
    if (it == g_cache.end()) return false;
    *choice = it->second;
    return true;
}

void store(const std::string &bucket, int choice) {
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    const std::string key = device_tag() + "|" + bucket;
    g_cache[key] = choice;
    const std::string path = cache_path();
    mkdirs(path);
    std::ofstream f(path, std::ios::app);
    if (f) f << key << "=" << choice << "\n";
}

} // namespace eg::autotune
