// engine.h — host runtime of the GB300 MD step: layout of the systems in HBM,
// device buffers, the captured step graph with its on-device rebuild
// decision, and recovery from capacity overflow.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "hmd_device.cuh"
#include "halmd_gb300.h"
#include "kernels.h"

namespace hmd {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char* what);
#define HMD_CUDA(x) ::hmd::cuda_check((x), #x)

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void alloc(size_t count)
    {
        release();
        if (count == 0) return;
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            (void)cudaGetLastError();
            throw Error(HMD_ERR_NOMEM, std::string("device allocation of ") + std::to_string(count * sizeof(T)) +
                                           " bytes failed: " + cudaGetErrorString(e));
        }
        n = count;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

struct SysHost {
    hmd_system_desc desc;
    SysParam P;
    std::vector<PairParam> pairs;
    std::vector<PairParam64> pairs64;   // the same table in double (FP64 variant)
    uint32_t nbr_size = 0;   // list capacity estimate (from_binning.cpp:96-119)
    bool used = false;       // the table entry holds a system
};

// first-fit allocator of [0, cap) in fixed units (slot tiles, cells, cell words)
class Arena {
public:
    void init(uint32_t cap)
    {
        free_.clear();
        used_ = 0;
        if (cap) free_[0] = cap;
    }
    bool alloc(uint32_t n, uint32_t& at);
    void release(uint32_t at, uint32_t n);
    uint32_t used() const { return used_; }

private:
    std::map<uint32_t, uint32_t> free_;   // start -> length
    uint32_t used_ = 0;
};

class Engine {
public:
    Engine(int precision, int device);
    ~Engine();

    uint32_t add_system(const hmd_system_desc& desc);
    void reserve(uint32_t slots, uint32_t systems, uint32_t neighbour_capacity);
    void commit();
    void remove_system(uint32_t s);
    void capacity_info(uint64_t* out) const;
    void progress(uint64_t* step, uint32_t* steps_left, uint32_t n);
    uint64_t bytes_per_slot() const;
    void set(uint32_t s, const std::string& name, const void* host, size_t count);
    void get(uint32_t s, const std::string& name, void* host, size_t count);
    void get_raw(uint32_t s, const std::string& name, void* host, size_t bytes);
    void info(uint32_t s, hmd_system_info* out);

    void step(uint64_t nsteps, bool aux_last);
    void integrate();
    void force(bool aux);
    void finalize();
    void request_rebuild(uint32_t s);
    void set_steps_left(uint32_t s, uint32_t steps);
    void minimize(uint32_t s, uint32_t steps, double step_size, double max_move);
    uint32_t block() const;
    void stage(size_t doubles);
    void set_option(const std::string& name, int64_t value);
    int64_t get_option(const std::string& name) const;
    double max_displacement(uint32_t s);
    void thermo(uint32_t s, double* out);
    void integrator_state(uint32_t s, double* out);
    void lattice(uint32_t s, const double* slab);
    void boltzmann(uint32_t s, double temperature, uint64_t seed);
    void neighbour_lists(uint32_t s, uint32_t* counts, uint32_t* lists, uint32_t maxn);
    void hilbert_keys(uint32_t s, uint32_t* keys);
    void profile_enable(bool on);
    void profile_get(const std::string& phase, double* total_ms, uint64_t* count);

    // used by the dynamics module
    Dev dev() const;
    cudaStream_t stream() const { return stream_; }
    const SysHost& system(uint32_t s) const;
    uint32_t nsys() const { return (uint32_t)sys_.size(); }
    uint32_t slots() const { return S_; }
    // dsfloat storage (hi + lo words): the dsfloat engines and the FP64 variant
    bool ds() const { return precision_ == HMD_PRECISION_DSFLOAT || precision_ == HMD_PRECISION_DOUBLE; }
    bool fp64() const { return precision_ == HMD_PRECISION_DOUBLE; }
    void sync();

    std::string err;

private:
    void check_committed() const;
    void check_sys(uint32_t s) const;
    void layout_system(SysHost& h, uint32_t rank, uint32_t align);
    void upload_tables();
    void upload_system(uint32_t s);
    void install(uint32_t s);
    bool place(uint32_t s);
    void unplace(uint32_t s);
    uint32_t add_live_system(const hmd_system_desc& desc);
    void ensure_forces(bool aux);
    void rebuild_chain(cudaStream_t st);
    void build_graphs();
    void destroy_graphs();
    cudaGraphExec_t capture(int nsteps, bool aux_last);
    bool fused() const;
    uint64_t chunk_kernels(int n) const;
    void snapshot();
    void restore();
    bool grow_after_overflow(uint32_t status);
    void run_steps(uint64_t nsteps, bool aux_last);
    std::vector<SysState> read_state();
    void write_state(const std::vector<SysState>& st);
    template <typename T> void download(const DevBuf<T>& b, size_t first, size_t count, T* host);
    template <typename T> void upload(DevBuf<T>& b, size_t first, size_t count, const T* host);
    // the hi (lo = false) or lo words of slots [first, first + count) of the
    // interleaved position array (hmd_device.cuh), as a packed float4 array
    void download_pos(bool lo, size_t first, size_t count, float4* host);
    void upload_pos(bool lo, size_t first, size_t count, const float4* host);
    std::vector<uint32_t> slots_of(uint32_t s);   // slot (absolute) of each tag

    int precision_;
    int device_;
    bool committed_ = false;
    bool forces_valid_ = false;
    bool aux_valid_ = false;
    bool integrated_ = false;   // hmd_integrate since the last force
    std::vector<SysHost> sys_;
    uint32_t table_size_ = 0;      // entries of the device system tables
    uint32_t null_sys_ = 0xFFFFFFFFu;   // inert owner of free ranges (capacity mode)
    bool capacity_ = false;
    uint32_t cap_slots_ = 0, cap_systems_ = 0, cap_nbr_ = 0;
    Arena slot_arena_, cell_arena_, word_arena_;
    uint32_t S_ = 0;
    uint32_t total_cells_ = 0;
    uint32_t nbr_cap_ = 0;
    uint32_t lanes_ = 0;        // force-kernel lanes per particle (0: choose at commit)
    uint32_t lb_ = 0;          // list block width option (0 auto, 4, 8)
    uint32_t nbr_scan_ = 0;   // list build: 0 auto, 1 per lane, 2 shared scan per warp
    uint32_t sm_count_ = 0;   // SMs of the device
    uint32_t grid_slots_ = 0, grid_cells_ = 0;   // launch-grid extents (update_grid_extent)
    void update_grid_extent();
    uint32_t force_kinds_ = 0;  // Dev::force_kinds: kinds of the committed systems (0 in capacity mode)
    uint32_t integ_kinds_ = 0;  // Dev::integ_kinds: integrators of the committed systems
    int sort_passes_ = 0;       // radix passes of the segmented sort (even)
    uint32_t ntiles_ = 0;
    DevBuf<uint2> tiles_;
    uint32_t key_bits_ = 0;
    bool any_sort_ = false;
    cudaStream_t stream_ = nullptr;
    cudaStream_t side_ = nullptr;

    DevBuf<float4> pos_, vel_, img_, force_, r0_, tpos_, tvel_, timg_;
    DevBuf<float4> fpos_;   // dsfloat engines: the force kernel's gather records
    DevBuf<Force64> force64_, snap_force64_;   // FP64 variant: forces in double
    DevBuf<PairParam64> dpair64_;
    DevBuf<float> en_pot_, stress_;
    DevBuf<uint32_t> id_, rid_, nbr_, nbr_count_, cell_, cell_count_, cell_sys_, chunk_sys_, tid_;
    DevBuf<uint32_t> key0_, key1_, val0_, val1_, hist_, dtot_, status_, done_, any_rebuild_, rb_;
    DevBuf<SysParam> dsys_;
    DevBuf<SysState> dst_;
    DevBuf<PairParam> dpair_;
    DevBuf<double> partial_, thermo_;
    DevBuf<double> io_;                          // staging of tag-ordered set / get arrays
    // overflow snapshot
    DevBuf<float4> snap_pos_, snap_vel_, snap_img_, snap_force_;
    DevBuf<uint32_t> snap_id_, snap_rid_;
    DevBuf<SysState> snap_st_;

    // per-phase CUDA-event timers of the module-level calls
    struct Timer {
        double ms = 0;
        uint64_t count = 0;
    };
    bool profile_ = false;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    std::vector<std::pair<std::string, Timer>> timers_;
    void tic();
    void toc(const char* phase);
    uint32_t rebuild_kernel_count() const;

    static constexpr int CHUNK_STEPS = 100;
    static constexpr int SHORT_STEPS = 10;       // chunk for the remainder below CHUNK_STEPS
    static constexpr uint64_t SEGMENT_STEPS = 5000;
    cudaGraphExec_t g_chunk_ = nullptr, g_short_ = nullptr, g_one_ = nullptr, g_one_aux_ = nullptr;
    bool fuse_ = true;                           // captured chunks fuse finalize k with integrate k+1
    bool float_cutoff_ = false;                  // FP64 variant: float cut-off decision (set_option)
    uint64_t step_kernels_ = 0;                  // kernels of the step graphs launched (rebuild chains not counted)
};

} // namespace hmd
