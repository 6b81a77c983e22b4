// dynamics.h — blocking scheme and time-correlation functions (MSD, MQD,
// VACF, ISF) over one system of an engine.
//   blocking scheme   observables/dynamics/blocking_scheme.cpp:35-200,
//                     observables/samples/blocking_scheme.hpp:74-189
//   correlation       observables/dynamics/correlation.hpp:208-224
//   MSD               observables/gpu/dynamics/mean_square_displacement.cpp:55-68
//   MQD               observables/dynamics/mean_quartic_displacement.hpp:34-41
//   VACF              observables/dynamics/velocity_autocorrelation.hpp:34-38
//   ISF               observables/dynamics/intermediate_scattering_function.hpp:89-113
//   wavevectors       observables/utility/wavevector.cpp:40-160,
//                     algorithm/host/pick_lattice_points.hpp:74-160
#pragma once

#include <deque>
#include <memory>
#include <vector>

#include "engine.h"

namespace hmd {

struct Accum {
    double n = 0, m = 0, v = 0;   // count, mean, variance x count
    void merge(double n2, double m2, double v2);
    void add(double x);
};

class Dynamics {
public:
    Dynamics(Engine& e, uint32_t sys, double max_lag_time, double resolution, uint32_t block_size, uint32_t shift,
             uint32_t separation);
    uint32_t levels() const { return (uint32_t)interval_.size(); }
    uint32_t block_size() const { return block_size_; }
    void time(double* out) const;
    int32_t add_msd(uint32_t first, uint32_t last) { return add_particle_tcf(0, first, last); }
    int32_t add_mqd(uint32_t first, uint32_t last) { return add_particle_tcf(2, first, last); }
    int32_t add_vacf(uint32_t first, uint32_t last) { return add_particle_tcf(3, first, last); }
    int32_t add_isf(const double* wavenumber, uint32_t nk, double tolerance, uint32_t max_count, uint32_t first,
                    uint32_t last, double norm);
    void sample();
    void finalise();
    void result(int32_t tcf, double* mean, double* error, uint64_t* count) const;
    void shells(int32_t tcf, uint32_t* nshell, double* wavenumber) const;

private:
    struct Rho {
        std::vector<double> v;   // (re, im) per wavevector
    };
    struct PosSample {
        DevBuf<double> r;        // unwrapped positions, tag order, 3n
    };
    struct Sample {
        uint64_t step = 0;
        std::shared_ptr<PosSample> pos;
        std::shared_ptr<PosSample> vel;          // velocities, tag order, 3n (VACF)
        std::vector<std::shared_ptr<Rho>> rho;   // per ISF
    };
    struct Tcf {
        int kind = 0;            // 0: MSD, 1: ISF, 2: MQD, 3: VACF
        uint32_t first = 0, last = 0;
        double norm = 1;
        int isf = -1;            // index into Sample::rho
        uint32_t nshell = 1;
        std::vector<double> wavenumber;
        std::vector<uint32_t> shell;   // [2*nshell] wavevector index ranges
        uint32_t nq = 0;
        DevBuf<float4> q;
        std::vector<Accum> res;  // [levels * block_size * nshell]
        // device scratch of the group reduction
        DevBuf<uint32_t> range, blk_range, blk_begin;
        uint32_t nblk = 0;
        DevBuf<double> partial, out;
    };

    int32_t add_particle_tcf(int kind, uint32_t first, uint32_t last);
    uint64_t current_step();
    std::shared_ptr<Sample> acquire(uint64_t step);
    void process(uint32_t level);
    void correlate(Tcf& t, const Sample& a, const Sample& b, Accum* out);
    void setup_blocks(Tcf& t, uint32_t begin, uint32_t end, uint32_t chunk);

    Engine& e_;
    uint32_t sys_;
    double dt_;
    uint32_t block_size_, separation_;
    std::vector<uint64_t> interval_, origin_;
    std::vector<std::deque<std::shared_ptr<Sample>>> blocks_;
    std::vector<std::unique_ptr<Tcf>> tcf_;
    std::shared_ptr<Sample> last_;
    bool started_ = false;
};

} // namespace hmd
