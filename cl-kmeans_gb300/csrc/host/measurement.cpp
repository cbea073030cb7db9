// Measurement CSV writer (schema of measurement/measurement.cpp:203-366).
#include "measurement.hpp"

#include <unistd.h>

#include <chrono>
#include <ctime>
#include <fstream>
#include <random>
#include <sstream>

namespace Measurement {

static const uint32_t max_datetime_length = 30;
static const char* const timestamp_format = "%F-%H-%M-%S";
static const char* const experiment_file_suffix = "_expm";
static const char* const measurements_file_suffix = "_mnts";
static const char* const events_file_suffix = "_evnt";

uint64_t DataPoint::get_value() {
    uint64_t value = 0;
    if (has_event_ && !events_.empty()) {
        for (const Event& e : events_) value += e.duration_ns();
    } else {
        for (uint64_t v : values_) value += v;
    }
    for (auto& child : children_) value += child.get_value();
    return value;
}

uint64_t DataPoint::get_event_queued(size_t i) {
    if (!has_event_ || i >= events_.size()) return 0;
    return events_[i].queued_ns();
}

uint64_t DataPoint::get_event_submit(size_t i) {
    // CUDA exposes no separate submit timestamp; it equals the enqueue time.
    return get_event_queued(i);
}

uint64_t DataPoint::get_event_start(size_t i) {
    if (!has_event_ || i >= events_.size()) return 0;
    if (!origin_ || !origin_->valid()) return events_[i].queued_ns();
    return (uint64_t)((int64_t)origin_host_ns_ + events_[i].start_since(origin_->end_event()));
}

uint64_t DataPoint::get_event_end(size_t i) {
    if (!has_event_ || i >= events_.size()) return 0;
    if (!origin_ || !origin_->valid()) return events_[i].queued_ns() + events_[i].duration_ns();
    return (uint64_t)((int64_t)origin_host_ns_ + events_[i].end_since(origin_->end_event()));
}

uint64_t DataPoint::get_event_queue_id(size_t i) {
    if (!has_event_ || i >= events_.size()) return 0;
    return events_[i].queue_id();
}

Measurement::Measurement() : run_(0), origin_host_ns_(0) {
    run_date_ = std::chrono::system_clock::now();
    set_parameter("TimeStamp", get_datetime());
}

Measurement::~Measurement() {}

void Measurement::set_run(int run) { run_ = run; }

void Measurement::set_parameter(std::string name, std::string value) { parameters_[name] = value; }

std::string Measurement::get_parameter(const std::string& name) const {
    auto it = parameters_.find(name);
    return it == parameters_.end() ? std::string() : it->second;
}

void Measurement::stamp(DataPoint& dp) {
    dp.origin_ = origin_;
    dp.origin_host_ns_ = origin_host_ns_;
}

DataPoint& Measurement::add_datapoint() {
    data_points_.push_back(DataPoint());
    stamp(data_points_.back());
    return data_points_.back();
}

DataPoint& Measurement::add_datapoint(int iteration) {
    data_points_.push_back(DataPoint(iteration));
    stamp(data_points_.back());
    return data_points_.back();
}

void Measurement::set_origin(const Clustering::Stream& queue) {
    origin_ = std::make_shared<Clustering::Event>(Clustering::Event::marker(queue));
    origin_->wait();
    origin_host_ns_ = Clustering::host_now_ns();
    for (auto& dp : data_points_) stamp(dp);
}

uint64_t Measurement::total_by_name(const std::string& name) {
    uint64_t t = 0;
    for (auto& dp : data_points_)
        if (dp.get_name() == name) t += dp.get_value();
    return t;
}

std::vector<std::string> Measurement::write_csv(std::string filename) {
    std::string experiment_id = get_unique_id();
    std::vector<std::string> paths;
    {
        std::string f = format_filename(filename, experiment_id, experiment_file_suffix);
        std::ofstream pf(f, std::ios_base::out | std::ios::trunc);
        pf << "ExperimentID" << ',' << "ParameterName" << ',' << "Value" << "\n";
        for (auto const& p : parameters_) pf << experiment_id << ',' << p.first << ',' << p.second << '\n';
        paths.push_back(f);
    }
    {
        std::string f = format_filename(filename, experiment_id, measurements_file_suffix);
        std::ofstream mf(f, std::ios_base::out | std::ios::trunc);
        mf << "ExperimentID" << ',' << "Run" << ',' << "TypeName" << ',' << "Iteration" << ',' << "Value" << '\n';
        for (DataPoint dp : get_flattened_datapoints()) {
            mf << experiment_id << ',' << run_ << ',' << dp.get_name() << ',';
            if (dp.is_iterative()) mf << dp.get_iteration();
            mf << ',' << dp.get_value() << '\n';
        }
        paths.push_back(f);
    }
    {
        std::string f = format_filename(filename, experiment_id, events_file_suffix);
        std::ofstream ef(f, std::ios_base::out | std::ios::trunc);
        ef << "ExperimentID" << ',' << "Run" << ',' << "TypeName" << ',' << "Iteration" << ',' << "CommandQueueID"
           << ',' << "Queued" << ',' << "Submit" << ',' << "Start" << ',' << "End" << '\n';
        for (DataPoint dp : get_datapoints_with_events()) {
            for (size_t i = 0; i < dp.num_events(); ++i) {
                ef << experiment_id << ',' << run_ << ',' << dp.get_name() << ',';
                if (dp.is_iterative()) ef << dp.get_iteration();
                ef << ',' << dp.get_event_queue_id(i) << ',' << dp.get_event_queued(i) << ','
                   << dp.get_event_submit(i) << ',' << dp.get_event_start(i) << ',' << dp.get_event_end(i) << '\n';
            }
        }
        paths.push_back(f);
    }
    return paths;
}

std::string Measurement::get_unique_id() {
    std::random_device rand;
    std::stringstream ss;
    ss << std::dec << rand();
    return ss.str();
}

std::string Measurement::get_datetime() {
    char datetime[max_datetime_length];
    std::time_t t = std::chrono::system_clock::to_time_t(run_date_);
    std::tm tmv;
    gmtime_r(&t, &tmv);
    std::strftime(datetime, max_datetime_length, timestamp_format, &tmv);
    return datetime;
}

// <parent>/<datetime>_<id>_<stem><suffix><extension>, like the reference's
// boost::filesystem composition (measurement.cpp:340-366).
std::string Measurement::format_filename(std::string base_file, std::string experiment_id, std::string suffix) {
    std::string parent, name = base_file;
    size_t slash = base_file.find_last_of('/');
    if (slash != std::string::npos) {
        parent = base_file.substr(0, slash);
        name = base_file.substr(slash + 1);
    }
    std::string stem = name, ext;
    size_t dot = name.find_last_of('.');
    if (dot != std::string::npos && dot != 0) {
        stem = name.substr(0, dot);
        ext = name.substr(dot);
    }
    std::string out = parent;
    if (!out.empty()) out += '/';
    out += get_datetime() + '_' + experiment_id + '_' + stem + suffix + ext;
    return out;
}

std::deque<DataPoint> Measurement::get_flattened_datapoints() {
    std::deque<DataPoint> sub;
    for (auto& dp : data_points_) {
        if (!dp.children_.empty()) {
            DataPoint cp = dp.is_iterative() ? DataPoint(dp.get_iteration()) : DataPoint();
            cp.set_name(dp.get_name() + "#Sub");
            uint64_t v = 0;
            for (auto& child : dp.children_) v += child.get_value();
            cp.add_value() = v;
            sub.push_back(cp);
        }
        sub.push_back(dp);
    }
    return sub;
}

std::deque<DataPoint> Measurement::get_datapoints_with_events() {
    std::deque<DataPoint> out;
    std::deque<DataPoint> stack(data_points_);
    while (!stack.empty()) {
        DataPoint dp = stack.front();
        stack.pop_front();
        if (dp.num_events() > 0) out.push_back(dp);
        for (auto& cp : dp.children_) {
            cp.origin_ = dp.origin_;
            cp.origin_host_ns_ = dp.origin_host_ns_;
            stack.push_front(cp);
        }
    }
    return out;
}

}  // namespace Measurement
