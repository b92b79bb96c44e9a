// run_loop.cu — the time loop with the reference's layer output.
//
// rrsph_run mirrors time_integration + RRSPHOutput
// (sources/RRSPH_OMP/src/TimeIntegration.cpp:53-100,
//  sources/RRSPH_COMMON/src/Output.cpp:28-79, 223-446):
//   - the first data layer is written at the start time (setup_output);
//   - the loop runs while time <= simulation_time; after each step
//     update_step writes data/<t>.csv when time - last_save_time > save_time
//     (or every step with save_every_step) and dump/<t>.csv when use_dump and
//     time - last_dump_time > dump_time;
//   - a consistency failure under CONSISTENCY_STOP writes crash_dump_<t>.csv
//     (use_crash_dump) and stops with the error.
// The steps between two layer times run as one batch of graph replays; the
// host predicts the batch length from the same double additions the device
// makes (time += dt), except under a true dynamic-dt reduction, where it
// steps one at a time. Layers are copied to pinned host buffers and formatted
// by a pool of writer threads while the GPU continues.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <filesystem>
#include <limits>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../host/error.hpp"
#include "solver_impl.cuh"

using rrsph::set_error;

namespace {

// format_count_decimal_digits / format_time_digits (RRSPH_COMMON/src/TimeFormat.cpp:36-53)
int count_decimal_digits(double val) {
    if (val > 10) return 0;
    if (val > 1) return 1;
    int count = 1;
    while (val < 1) {
        val *= 10;
        count++;
    }
    return count;
}
std::string time_digits(double time, int digits) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.*f", digits, time);
    return buf;
}

// One layer's arrays in one host block.
struct Block {
    char* data = nullptr;
    bool pinned = false;
};

// Host blocks for the layers in flight. Up to max_pinned of them are
// page-locked and kept for reuse (rrsph_download then writes them with one
// kernel over the host link); past that, pageable blocks are allocated and
// freed per layer (rrsph_download copies into them through a staging buffer).
class BlockPool {
public:
    BlockPool(size_t bytes, size_t max_pinned) : bytes_(bytes), max_pinned_(max_pinned) {}
    BlockPool(const BlockPool&) = delete;
    BlockPool& operator=(const BlockPool&) = delete;
    ~BlockPool() {
        for (const Block& b : free_) cudaFreeHost(b.data);
    }
    size_t bytes() const { return bytes_; }
    Block get() {
        {
            std::lock_guard<std::mutex> lock(mu_);
            if (!free_.empty()) {
                const Block b = free_.back();
                free_.pop_back();
                return b;
            }
            if (pinned_ < max_pinned_) {
                void* q = nullptr;
                if (cudaMallocHost(&q, bytes_) == cudaSuccess) {
                    pinned_++;
                    return {static_cast<char*>(q), true};
                }
                cudaGetLastError();
                max_pinned_ = pinned_;  // no more page-locked memory: stop asking
            }
        }
        return {static_cast<char*>(std::malloc(bytes_)), false};
    }
    void put(const Block& b) {
        if (!b.data) return;
        if (!b.pinned) {
            std::free(b.data);
            return;
        }
        std::lock_guard<std::mutex> lock(mu_);
        free_.push_back(b);
    }

private:
    const size_t bytes_;
    size_t max_pinned_;
    size_t pinned_ = 0;
    std::mutex mu_;
    std::vector<Block> free_;
};

// Byte offsets of the arrays in a block (16-byte aligned starts).
struct LayerShape {
    size_t n, dim, r, v, rho, p, itype, bytes;
    LayerShape(size_t n_, size_t dim_) : n(n_), dim(dim_) {
        auto up = [](size_t x) { return (x + 15) & ~size_t(15); };
        r = 0;
        v = up(r + n * dim * sizeof(double));
        rho = up(v + n * dim * sizeof(double));
        p = up(rho + n * sizeof(double));
        itype = up(p + n * sizeof(double));
        bytes = up(itype + n * sizeof(int32_t));
    }
};

// A layer on its way to a file: the arrays (in a pool block) and the path.
struct Layer {
    BlockPool* pool = nullptr;
    Block block;
    std::string path;
    bool dump = false;
    Layer() = default;
    Layer(const Layer&) = delete;
    Layer& operator=(const Layer&) = delete;
    Layer(Layer&& o) noexcept : pool(o.pool), block(o.block), path(std::move(o.path)), dump(o.dump) { o.block = {}; }
    Layer& operator=(Layer&& o) noexcept {
        if (this != &o) {
            release();
            pool = o.pool;
            block = o.block;
            path = std::move(o.path);
            dump = o.dump;
            o.block = {};
        }
        return *this;
    }
    ~Layer() { release(); }
    void release() {
        if (pool) pool->put(block);
        block = {};
    }
    double* f64(size_t off) const { return reinterpret_cast<double*>(block.data + off); }
    int32_t* i32(size_t off) const { return reinterpret_cast<int32_t*>(block.data + off); }
};

// Writer threads for the CSV layers.
class Writers {
public:
    Writers(const rrsph_params& p, const LayerShape& shape, unsigned n) : params_(p), shape_(shape) {
        for (unsigned i = 0; i < n; i++) threads_.emplace_back([this] { loop(); });
    }
    ~Writers() { finish(); }
    void push(Layer&& layer) {
        std::unique_lock<std::mutex> lock(mu_);
        room_.wait(lock, [this] { return queue_.size() < 8; });  // bound the host memory held
        queue_.push_back(std::move(layer));
        cv_.notify_one();
    }
    // Waits for every queued layer; returns the first write error (RRSPH_OK if none).
    int finish() {
        {
            std::lock_guard<std::mutex> lock(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : threads_)
            if (t.joinable()) t.join();
        threads_.clear();
        return rc_;
    }
    const std::string& error() const { return err_; }

private:
    void loop() {
        for (;;) {
            Layer l;
            {
                std::unique_lock<std::mutex> lock(mu_);
                cv_.wait(lock, [this] { return stop_ || !queue_.empty(); });
                if (queue_.empty()) return;
                l = std::move(queue_.front());
                queue_.pop_front();
                room_.notify_one();
            }
            const int rc = rrsph_layer_write(l.path.c_str(), &params_, l.f64(shape_.r), params_.dim,
                                             l.f64(shape_.v), l.f64(shape_.rho), l.f64(shape_.p),
                                             l.i32(shape_.itype), l.dump ? 1 : 0);
            l.release();  // before the next layer is taken
            if (rc) {
                std::lock_guard<std::mutex> lock(mu_);
                if (!rc_) {
                    rc_ = rc;
                    err_ = rrsph_last_error();
                }
            }
        }
    }
    rrsph_params params_;
    LayerShape shape_;
    std::mutex mu_;
    std::condition_variable cv_, room_;
    std::deque<Layer> queue_;
    std::vector<std::thread> threads_;
    bool stop_ = false;
    int rc_ = RRSPH_OK;
    std::string err_;
};

// The current state into a fresh layer from the pool.
int snapshot(rrsph_solver* s, BlockPool& pool, const LayerShape& sh, Layer& l) {
    l.release();
    l.pool = &pool;
    l.block = pool.get();
    if (!l.block.data) return set_error(RRSPH_ERR_OUT_OF_MEMORY, "rrsph_run: no host memory for a layer");
    return rrsph_download(s, l.f64(sh.r), (uint32_t)sh.dim, l.f64(sh.v), l.f64(sh.rho), l.f64(sh.p),
                          l.i32(sh.itype));
}

// A second layer with the same arrays.
int copy_layer(BlockPool& pool, const LayerShape& sh, const Layer& from, Layer& to) {
    to.release();
    to.pool = &pool;
    to.block = pool.get();
    if (!to.block.data) return set_error(RRSPH_ERR_OUT_OF_MEMORY, "rrsph_run: no host memory for a layer");
    std::memcpy(to.block.data, from.block.data, sh.bytes);
    return RRSPH_OK;
}

}  // namespace

extern "C" int rrsph_run(rrsph_solver* s, const char* experiment_dir, double* time_io, uint64_t max_steps,
                         uint64_t* steps_done) {
    if (!s || !experiment_dir || !time_io) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_run: null argument");
    namespace fs = std::filesystem;
    const rrsph_params& p = s->params;
    const fs::path dir(experiment_dir);
    std::error_code ec;
    if (!fs::is_directory(dir, ec))
        return set_error(RRSPH_ERR_IO, "No experiment directory exists: " + dir.string());
    fs::create_directories(dir / "data", ec);
    fs::create_directories(dir / "dump", ec);
    const int save_digits = count_decimal_digits(p.save_time);
    const int dump_digits = count_decimal_digits(p.dump_time);
    // dt the device will use for every step, when it is known in advance
    const bool stepwise = p.dt_correction_method == 2 && p.dt_dynamic_reduce;
    double dt = p.dt;
    if (p.dt_correction_method == 2 && !p.dt_dynamic_reduce) {
        const double c_sqr = p.eos_sound_vel_method == 0 ? 200 * p.g * p.depth * p.eos_sound_vel_coef : p.eos_sound_vel;
        // update_dt(0, 0) of the OMP build: sqrt(h / 0) is +inf, so the sound speed decides
        dt = p.CFL_coef * std::min(std::numeric_limits<double>::infinity(), p.hsml / (std::sqrt(c_sqr) + 0.0));
    }
    const unsigned nthreads = std::max(1u, std::min(8u, std::thread::hardware_concurrency() / 2));
    const LayerShape shape(p.ntotal, p.dim);
    // page-locked blocks for the layers in flight, up to 1 GiB (at least two)
    BlockPool pool(shape.bytes, std::max<size_t>(2, (size_t(1) << 30) / std::max<size_t>(shape.bytes, 1)));
    Writers writers(p, shape, nthreads);  // after the pool: the writers finish before it goes

    double time = *time_io;
    double last_save = time, last_dump = time;
    uint64_t done = 0;
    int rc = RRSPH_OK;
    {   // first layer (setup_output)
        Layer l;
        if ((rc = snapshot(s, pool, shape, l)) != 0) return rc;
        l.path = (dir / "data" / (time_digits(time, save_digits) + ".csv")).string();
        writers.push(std::move(l));
    }
    while (time <= p.simulation_time && done < max_steps) {
        // steps up to and including the next one that writes a layer
        uint64_t k = 0;
        double t = time;
        bool save = false, dump = false;
        while (t <= p.simulation_time && done + k < max_steps) {
            t = t + dt;
            k++;
            save = p.save_every_step || (t - last_save) > p.save_time;
            dump = p.use_dump && (t - last_dump) > p.dump_time;
            if (save || dump || stepwise || k >= 1000) break;
        }
        if (k == 0) break;
        double tn = time;
        rc = rrsph_step(s, k, &tn);
        done += k;
        time = tn;
        if (stepwise) {  // the device chose dt: decide the layers from its time
            save = p.save_every_step || (time - last_save) > p.save_time;
            dump = p.use_dump && (time - last_dump) > p.dump_time;
        }
        if (rc == RRSPH_ERR_OUTSIDE_GEOMETRY) {
            if (p.use_crash_dump) {
                Layer l;
                if (snapshot(s, pool, shape, l) == RRSPH_OK) {
                    l.path = (dir / ("crash_dump_" + time_digits(time, save_digits) + ".csv")).string();
                    l.dump = true;
                    writers.push(std::move(l));
                }
            }
            break;
        }
        if (rc) break;
        if (save || dump) {
            Layer l;
            if ((rc = snapshot(s, pool, shape, l)) != 0) break;
            if (save && dump) {
                Layer d;
                if ((rc = copy_layer(pool, shape, l, d)) != 0) break;
                d.path = (dir / "dump" / (time_digits(time, dump_digits) + ".csv")).string();
                d.dump = true;
                writers.push(std::move(d));
            } else if (dump) {
                l.path = (dir / "dump" / (time_digits(time, dump_digits) + ".csv")).string();
                l.dump = true;
            }
            if (save) {
                l.path = (dir / "data" / (time_digits(time, save_digits) + ".csv")).string();
                l.dump = false;
            }
            writers.push(std::move(l));
            if (save) last_save = time;
            if (dump) last_dump = time;
        }
    }
    const int wrc = writers.finish();
    *time_io = time;
    if (steps_done) *steps_done = done;
    if (rc) return rc;
    if (wrc) return set_error(wrc, writers.error());
    return RRSPH_OK;
}
