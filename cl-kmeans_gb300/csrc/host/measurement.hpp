// Measurement: named, per-iteration timing data points with profiling
// events, written to the reference's three CSV files.  Same classes, methods
// and CSV schema as measurement/measurement.hpp:20-146 and
// measurement/measurement.cpp:203-366; events are CUDA event pairs instead of
// OpenCL profiling events.
#pragma once

#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <regex>
#include <string>
#include <tuple>
#include <vector>

#include "device.hpp"

namespace Measurement {

class Measurement;

class DataPoint {
    friend class Measurement;

public:
    using Event = Clustering::Event;

    DataPoint& set_name(std::string name) {
        name_ = std::move(name);
        return *this;
    }

    // Starts a profiling event pair on `queue`; close it with Event::record_end.
    Event& add_event(const Clustering::Stream& queue) {
        has_event_ = true;
        events_.push_back(Event::record_start(queue));
        return events_.back();
    }
    // Attaches an already recorded event pair.
    Event& add_event(const Event& e) {
        has_event_ = true;
        events_.push_back(e);
        return events_.back();
    }

    uint64_t& add_value() {
        values_.push_back(0);
        return values_.back();
    }

    DataPoint& create_child() {
        children_.push_back(DataPoint());
        return children_.back();
    }

    std::string get_name() const { return name_; }
    bool is_iterative() const { return iterative_; }
    int get_iteration() const { return iteration_; }
    uint64_t get_value();
    size_t num_events() const { return has_event_ ? events_.size() : 0; }
    uint64_t get_event_queued(size_t i);
    uint64_t get_event_submit(size_t i);
    uint64_t get_event_start(size_t i);
    uint64_t get_event_end(size_t i);
    uint64_t get_event_queue_id(size_t i);

    DataPoint() : iterative_(false), iteration_(0), has_event_(false) {}
    explicit DataPoint(int iteration) : iterative_(true), iteration_(iteration), has_event_(false) {}

private:
    std::string name_;
    bool iterative_;
    int iteration_;
    bool has_event_;
    std::deque<Event> events_;
    std::deque<uint64_t> values_;
    std::deque<DataPoint> children_;
    // device-clock origin for absolute event times (set by Measurement)
    std::shared_ptr<Event> origin_;
    uint64_t origin_host_ns_ = 0;
};

class Measurement {
public:
    Measurement();
    ~Measurement();

    void set_run(int run);
    void set_parameter(std::string name, std::string value);
    std::string get_parameter(const std::string& name) const;
    const std::map<std::string, std::string>& parameters() const { return parameters_; }

    DataPoint& add_datapoint();
    DataPoint& add_datapoint(int iteration);

    // Writes <dir>/<UTC datetime>_<id>_<stem>{_expm,_mnts,_evnt}<ext>.
    // Returns the three paths.
    std::vector<std::string> write_csv(std::string filename);

    // Sum of all data points with this exact name (ns).
    uint64_t total_by_name(const std::string& name);

    template <typename UnitT = std::chrono::nanoseconds>
    std::vector<std::tuple<std::string, uint64_t>> get_execution_times_by_name(std::regex expression) {
        std::vector<std::tuple<std::string, uint64_t>> times;
        for (auto& dp : get_datapoints_with_events()) {
            if (std::regex_match(dp.get_name(), expression)) {
                for (size_t i = 0; i < dp.num_events(); ++i) {
                    std::chrono::nanoseconds ns(dp.get_event_end(i) - dp.get_event_start(i));
                    times.push_back(std::make_tuple(dp.get_name(),
                                                    (uint64_t)std::chrono::duration_cast<UnitT>(ns).count()));
                }
            }
        }
        return times;
    }

    // Records the device-clock origin on `queue` (done by the strategies
    // before their timed loop); event times in the CSV are relative to it.
    void set_origin(const Clustering::Stream& queue);

private:
    std::string get_unique_id();
    std::string get_datetime();
    std::string format_filename(std::string basefile, std::string experiment_id, std::string suffix);
    std::deque<DataPoint> get_flattened_datapoints();
    std::deque<DataPoint> get_datapoints_with_events();
    void stamp(DataPoint& dp);

    int run_;
    std::deque<DataPoint> data_points_;
    std::map<std::string, std::string> parameters_;
    std::chrono::system_clock::time_point run_date_;
    std::shared_ptr<Clustering::Event> origin_;
    uint64_t origin_host_ns_;
};

}  // namespace Measurement
