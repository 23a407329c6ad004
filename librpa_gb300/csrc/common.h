// Shared host-side helpers of the GB300 RPA library: errors, CUDA checks,
// owning device buffers and a small wall-clock timer.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

namespace gb {

// Error type raised inside the library; the C ABI converts it to a recorded
// error string and a NaN / no-op return (never lets an exception escape).
struct Error : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

#define GB_FAIL(msg)                                                                  \
    throw ::gb::Error(std::string(__FILE__) + ":" + std::to_string(__LINE__) + ": " + \
                      std::string(msg))

#define GB_REQUIRE(cond, msg)      \
    do                             \
    {                              \
        if (!(cond)) GB_FAIL(msg); \
    } while (0)

#define GB_CUDA(call)                                                                   \
    do                                                                                  \
    {                                                                                   \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            GB_FAIL(std::string("CUDA error ") + cudaGetErrorName(e_) + " (" +          \
                    cudaGetErrorString(e_) + ") in " #call);                            \
    } while (0)

// Checks the last launch; launches are asynchronous, so a fault inside a
// kernel surfaces at the next synchronising call, which GB_CUDA also checks.
#define GB_LAUNCH_CHECK() GB_CUDA(cudaGetLastError())

// Owning device allocation (cudaMalloc / cudaFree), move-only.
template <typename T>
class DevBuf
{
public:
    DevBuf() = default;
    explicit DevBuf(size_t n) { alloc(n); }
    ~DevBuf() { release(); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o)
        {
            release();
            p_ = o.p_; n_ = o.n_;
            o.p_ = nullptr; o.n_ = 0;
        }
        return *this;
    }
    void alloc(size_t n)
    {
        release();
        if (n == 0) return;
        GB_CUDA(cudaMalloc(&p_, n * sizeof(T)));
        n_ = n;
    }
    void release()
    {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }
    void zero(cudaStream_t s = 0)
    {
        if (p_) GB_CUDA(cudaMemsetAsync(p_, 0, n_ * sizeof(T), s));
    }
    void upload(const T *h, size_t n, cudaStream_t s = 0)
    {
        GB_REQUIRE(n <= n_, "upload larger than device buffer");
        if (n) GB_CUDA(cudaMemcpyAsync(p_, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void download(T *h, size_t n, cudaStream_t s = 0) const
    {
        GB_REQUIRE(n <= n_, "download larger than device buffer");
        if (n) GB_CUDA(cudaMemcpyAsync(h, p_, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    T *get() const { return p_; }
    size_t size() const { return n_; }
    size_t bytes() const { return n_ * sizeof(T); }

private:
    T *p_ = nullptr;
    size_t n_ = 0;
};

// A device copy of a host vector, staged on stream st.
template <typename T>
DevBuf<T> to_dev(const std::vector<T> &h, cudaStream_t st)
{
    DevBuf<T> d(h.size());
    d.upload(h.data(), h.size(), st);
    return d;
}

// Per-device one-time set-up (kernel attributes act on the current device only).  The
// caller keeps one PerDeviceOnce per set-up step; run() calls f() the first time it is used
// with a given device current, and is safe to call from several host threads.
class PerDeviceOnce
{
public:
    template <typename F>
    void run(F &&f)
    {
        int dev = -1;
        GB_CUDA(cudaGetDevice(&dev));
        GB_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal out of range");
        std::lock_guard<std::mutex> lk(mu_);
        if (done_[dev]) return;
        f();
        done_[dev] = true;
    }

private:
    static constexpr int kMaxDevices = 64;
    std::mutex mu_;
    bool done_[kMaxDevices] = {};
};

inline double wall_seconds()
{
    using clk = std::chrono::steady_clock;
    return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

} // namespace gb
