// Shim for the reference's missing MT data header, used ONLY to compile the
// reference's forward-solver sources as a test oracle (oracle/_ref).
//
// The reference's include/maple3dmt/data/ directory is not in its tree (its
// .gitignore rule `data/` also drops src/data and include/maple3dmt/data).
// These types are reconstructed from how the solve path and its callers use
// them: Station fields (examples/halfspace_1d_test.cpp:113-118), Datum with
// value/error/weight where unset components carry weight 0 and are skipped
// (src/inversion/inversion_fv.cpp:263-266), MTResponse with six Datum
// (src/utils/freq_parallel.cpp:175-189) and the MTData accessors called by
// src/forward/forward_solver_fv.cpp:68,1397-1398,1725,1736.
#pragma once

#include "maple3dmt/common.h"
#include <array>
#include <string>

namespace maple3dmt {
namespace data {

struct Station {
    std::string name;
    Real x = 0, y = 0, z = 0;
    Real lat = 0, lon = 0;
};

struct Datum {
    Complex value{0, 0};
    Real error = 0;
    Real weight = 0;
};

struct MTResponse {
    Datum Zxx, Zxy, Zyx, Zyy, Tx, Ty;
};

class MTData {
public:
    void add_station(const Station& s) {
        stations_.push_back(s);
        resize_();
    }
    const Station& station(int i) const { return stations_[i]; }
    Station& station_mut(int i) { return stations_[i]; }
    int num_stations() const { return static_cast<int>(stations_.size()); }

    void set_frequencies(const RealVec& f) {
        freqs_ = f;
        resize_();
    }
    const RealVec& frequencies() const { return freqs_; }
    int num_frequencies() const { return static_cast<int>(freqs_.size()); }

    const MTResponse& observed(int s, int f) const { return obs_[idx_(s, f)]; }
    const MTResponse& predicted(int s, int f) const { return pred_[idx_(s, f)]; }
    void set_observed(int s, int f, const MTResponse& r) { obs_[idx_(s, f)] = r; }
    void set_predicted(int s, int f, const MTResponse& r) { pred_[idx_(s, f)] = r; }

private:
    std::vector<Station> stations_;
    RealVec freqs_;
    std::vector<MTResponse> obs_, pred_;
    size_t idx_(int s, int f) const { return (size_t)s * freqs_.size() + (size_t)f; }
    void resize_() {
        obs_.resize(stations_.size() * freqs_.size());
        pred_.resize(stations_.size() * freqs_.size());
    }
};

}  // namespace data
}  // namespace maple3dmt
