// ckm_bench: the reference's `bench` driver (bench.cpp:46-510,
// clustering_benchmark.cpp:20-374) on the GB300 library.
//
//   ckm_bench --config X.conf [--csv out.csv] [--runs N] [--verify] [--verbose] FILE
//
// Same options, same .conf keys, same binary input, same three CSV files per
// run (parameters _expm, data points _mnts, events _evnt) with the same
// extra parameters (Version, Filename, Hostname, NumFeatures, NumPoints,
// NumClusters).  As in the reference, --k and --iterations are accepted but
// the .conf decides (bench.cpp:209-218).
//
// --verify runs a single-threaded CPU Lloyd (the reference's KmeansNaive
// arithmetic, verification only: it never produces the tool's results) and
// prints the number of differing labels and the centroid MSE
// (clustering_benchmark.cpp:276-326).
//
// Added: --generate OUT with --points/--features/--blobs/--seed/--sigma-lo/
// --sigma-hi writes a seeded Gaussian-mixture file with the device generator.
#include <unistd.h>

#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <iostream>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "../../../include/ckm.h"
#include "binary_format.hpp"
#include "configuration.hpp"
#include "kmeans_buffered.hpp"
#include "kmeans_single_stage.hpp"
#include "kmeans_three_stage.hpp"
#include "verify_naive.hpp"

#ifndef CKM_VERSION_STRING
#define CKM_VERSION_STRING "ckm-1.0"
#endif

using namespace Clustering;

namespace {

class CmdOptions {
public:
    int parse(int argc, char** argv) {
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i];
            auto value = [&](const char* name) -> std::string {
                if (i + 1 >= argc) throw std::invalid_argument(std::string("missing value for ") + name);
                return argv[++i];
            };
            auto eq = a.find('=');
            std::string key = a, inl;
            if (a.rfind("--", 0) == 0 && eq != std::string::npos) {
                key = a.substr(0, eq);
                inl = a.substr(eq + 1);
            }
            auto take = [&](const char* name) { return inl.empty() ? value(name) : inl; };
            if (key == "--help") {
                help_ = true;
            } else if (key == "--verbose") {
                verbose_ = true;
            } else if (key == "--verify") {
                verify_ = true;
            } else if (key == "--runs") {
                runs_ = (uint32_t)std::stoul(take("--runs"));
            } else if (key == "--k") {
                k_ = (uint32_t)std::stoul(take("--k"));
            } else if (key == "--iterations") {
                iterations_ = (uint32_t)std::stoul(take("--iterations"));
            } else if (key == "--csv") {
                csv_file_ = take("--csv");
            } else if (key == "--config") {
                config_file_ = take("--config");
            } else if (key == "--print-config") {
                print_config_ = true;
            } else if (key == "--info") {
                info_ = true;
            } else if (key == "--generate") {
                generate_ = take("--generate");
            } else if (key == "--points") {
                gen_points_ = std::stoull(take("--points"));
            } else if (key == "--features") {
                gen_features_ = (uint32_t)std::stoul(take("--features"));
            } else if (key == "--blobs") {
                gen_blobs_ = (uint32_t)std::stoul(take("--blobs"));
            } else if (key == "--seed") {
                gen_seed_ = std::stoull(take("--seed"));
            } else if (key == "--sigma-lo") {
                sigma_lo_ = std::stof(take("--sigma-lo"));
            } else if (key == "--sigma-hi") {
                sigma_hi_ = std::stof(take("--sigma-hi"));
            } else if (key == "--transfer") {
                transfer_ = true;
            } else if (key == "--max-size") {
                max_size_mib_ = std::stoull(take("--max-size"));
            } else if (key == "--repeat") {
                repeat_ = (uint32_t)std::stoul(take("--repeat"));
            } else if (key == "--device") {
                device_ = std::stoi(take("--device"));
            } else if (!a.empty() && a[0] == '-') {
                throw std::invalid_argument("unrecognised option '" + a + "'");
            } else {
                input_file_ = a;
            }
        }
        if (help_) {
            std::cout << "Usage: ckm_bench [OPTION] [FILE]\nOptions:\n"
                         "  --help                Produce help message\n"
                         "  --verbose             Show additional information\n"
                         "  --runs arg            Number of runs\n"
                         "  --k arg               Number of Clusters (the .conf decides)\n"
                         "  --iterations arg      Number of iterations (the .conf decides)\n"
                         "  --verify              Do verification pass\n"
                         "  --csv arg             Output measurements to CSV file\n"
                         "  --config arg          Configuration file\n"
                         "  --generate OUT        Write a seeded mixture file (--points --features --blobs\n"
                         "                        --seed --sigma-lo --sigma-hi)\n"
                         "  --print-config        Print the parsed configuration (one key=value per line)\n"
                         "  --info                Print the header of the input file\n"
                         "  --transfer            Host<->device link probe (--max-size MiB, default 256;\n"
                         "                        --repeat copies per size, default 10; --device)\n";
            return -1;
        }
        if (!generate_.empty() || transfer_) return 1;
        if (info_) {
            if (input_file_.empty()) {
                std::cout << "No input file specified." << std::endl;
                return -1;
            }
            return 1;
        }
        if (print_config_) {
            if (config_file_.empty()) {
                std::cout << "No config file specified." << std::endl;
                return -1;
            }
            return 1;
        }
        if (input_file_.empty()) {
            std::cout << "No input file specified." << std::endl;
            return -1;
        }
        if (config_file_.empty()) {
            std::cout << "No config file specified." << std::endl;
            return -1;
        }
        return 1;
    }

    bool help_ = false, verbose_ = false, verify_ = false, print_config_ = false, info_ = false;
    uint32_t k_ = 0, runs_ = 0, iterations_ = 0;
    std::string input_file_, csv_file_, config_file_, generate_;
    uint64_t gen_points_ = 1 << 20, gen_seed_ = 42;
    uint32_t gen_features_ = 4, gen_blobs_ = 10;
    float sigma_lo_ = 1.0f, sigma_hi_ = 1.0f;
    bool transfer_ = false;
    uint64_t max_size_mib_ = 256;
    uint32_t repeat_ = 10;
    int device_ = 0;
};

// --transfer: the link probe for chunk sizes 1 MiB .. --max-size MiB
// (doubling), both directions, pinned and pageable host memory.
int transfer_bench(const CmdOptions& o) {
    std::cout << "direction,host_memory,chunk_mib,repeat,best_gbs,mean_gbs" << std::endl;
    for (uint64_t mib = 1; mib <= std::max<uint64_t>(o.max_size_mib_, 1); mib *= 2) {
        for (int to_device = 1; to_device >= 0; --to_device) {
            for (int pinned = 1; pinned >= 0; --pinned) {
                double best = 0.0, mean = 0.0;
                const int rc = ckm_transfer_probe(o.device_, mib << 20, std::max<uint32_t>(o.repeat_, 1), pinned,
                                                  to_device, 3, &best, &mean);
                if (rc != CKM_OK) {
                    std::cerr << "ckm_bench: transfer probe failed: " << ckm_last_error() << std::endl;
                    return -1;
                }
                std::printf("%s,%s,%llu,%u,%.2f,%.2f\n", to_device ? "H2D" : "D2H", pinned ? "pinned" : "pageable",
                            (unsigned long long)mib, std::max<uint32_t>(o.repeat_, 1), best, mean);
            }
        }
    }
    return 1;
}

void first_x(const std::vector<float>& pts, size_t n, size_t d, size_t k, std::vector<float>& C) {
    for (size_t f = 0; f < d; ++f)
        for (size_t c = 0; c < k; ++c) C[f * k + c] = pts[f * n + (c % n)];
}
void first_x(const std::vector<double>& pts, size_t n, size_t d, size_t k, std::vector<double>& C) {
    for (size_t f = 0; f < d; ++f)
        for (size_t c = 0; c < k; ++c) C[f * k + c] = pts[f * n + (c % n)];
}

struct BenchStats {
    std::vector<uint64_t> microseconds;
    std::vector<std::shared_ptr<Measurement::Measurement>> measurements;
    uint64_t num_features = 0, num_points = 0, num_clusters = 0;

    void print_times(uint32_t runs) const {
        std::cout << runs << " runs, in µs: [";
        for (size_t r = 0; r < microseconds.size(); ++r) {
            std::cout << microseconds[r];
            if (r + 1 != microseconds.size()) std::cout << ", ";
        }
        std::cout << "]" << std::endl;
    }

    void to_csv(const std::string& csv_file, const std::string& input_file) {
        char hostname[64] = {0};
        gethostname(hostname, sizeof(hostname) - 1);
        std::string fname = input_file.substr(input_file.find_last_of('/') + 1);
        for (auto& m : measurements) {
            m->set_parameter("Version", CKM_VERSION_STRING);
            m->set_parameter("Filename", fname);
            m->set_parameter("Hostname", hostname);
            m->set_parameter("NumFeatures", std::to_string(num_features));
            m->set_parameter("NumPoints", std::to_string(num_points));
            m->set_parameter("NumClusters", std::to_string(num_clusters));
            for (const auto& path : m->write_csv(csv_file)) std::cout << "wrote " << path << std::endl;
        }
    }
};

template <typename P, typename L, typename M>
int run_bench(const CmdOptions& opt, const ConfigurationParser& config) {
    auto bm = config.get_benchmark_configuration();
    auto km = config.get_kmeans_configuration();
    auto gb = config.get_gb300_configuration();
    uint32_t runs = opt.runs_ ? opt.runs_ : (uint32_t)bm.runs;
    const bool verify = opt.verify_ || bm.verify;

    std::vector<P> points;
    uint64_t n = 0, d = 0;
    BinaryFormat bf;
    bf.read(opt.input_file_, points, n, d);
    const size_t k = km.clusters;
    if (k == 0 || d == 0) throw std::invalid_argument("kmeans.clusters and the file's features must be >= 1");
    auto sp = std::make_shared<const std::vector<P>>(std::move(points));

    using Fn = std::function<std::shared_ptr<Measurement::Measurement>(
        size_t, size_t, std::shared_ptr<const std::vector<P>>, std::shared_ptr<std::vector<P>>,
        std::shared_ptr<std::vector<M>>, std::shared_ptr<std::vector<L>>)>;
    Fn kmeans;
    const std::string& pipe = km.pipeline;
    auto pick_device = [](size_t dev) { cuda_check(cudaSetDevice((int)dev), "cudaSetDevice"); };
    if (pipe == "three_stage" || pipe == "three_stage_buffered") {
        auto ll = config.get_labeling_configuration();
        auto mu = config.get_mass_update_configuration();
        auto cu = config.get_centroid_update_configuration();
        pick_device(ll.device);
        if (pipe == "three_stage") {
            auto s = std::make_shared<KmeansThreeStage<P, L, M>>();
            Stream q_ll = Stream::create((int)ll.device);
            Stream q_mu = (mu.device == ll.device) ? q_ll : Stream::create((int)mu.device);
            Stream q_cu = (cu.device == ll.device) ? q_ll : ((cu.device == mu.device) ? q_mu : Stream::create((int)cu.device));
            s->set_labeling_queue(q_ll);
            s->set_mass_update_queue(q_mu);
            s->set_centroid_update_queue(q_cu);
            s->set_labeler(ll);
            s->set_mass_updater(mu);
            s->set_centroid_updater(cu);
            s->set_converge(km.converge);
            s->set_tolerance(gb.tolerance);
            s->set_spatial_order(gb.spatial_order);
            kmeans = [s](size_t a, size_t b, std::shared_ptr<const std::vector<P>> c, std::shared_ptr<std::vector<P>> e,
                         std::shared_ptr<std::vector<M>> f, std::shared_ptr<std::vector<L>> g) {
                return (*s)(a, b, c, e, f, g);
            };
        } else {
            auto s = std::make_shared<KmeansThreeStageBuffered<P, L, M>>();
            BufferedOptions bo;
            bo.device_budget_bytes = (uint64_t)gb.device_budget_mib << 20;
            bo.chunk_bytes = (uint64_t)gb.chunk_mib << 20;
            s->set_options(bo);
            s->set_labeler(ll);
            s->set_mass_updater(mu);
            s->set_centroid_updater(cu);
            s->set_converge(km.converge);
            s->set_tolerance(gb.tolerance);
            kmeans = [s](size_t a, size_t b, std::shared_ptr<const std::vector<P>> c, std::shared_ptr<std::vector<P>> e,
                         std::shared_ptr<std::vector<M>> f, std::shared_ptr<std::vector<L>> g) {
                return (*s)(a, b, c, e, f, g);
            };
        }
        if (opt.verbose_) {
            std::cout << "Labeling device: " << ll.device << std::endl
                      << "Mass update device: " << mu.device << std::endl
                      << "Centroid update device: " << cu.device << std::endl;
        }
    } else if (pipe == "single_stage" || pipe == "single_stage_buffered") {
        auto fu = config.get_fused_configuration();
        pick_device(fu.device);
        if (pipe == "single_stage") {
            auto s = std::make_shared<KmeansSingleStage<P, L, M>>();
            s->set_queue(Stream::create((int)fu.device));
            s->set_fused(fu);
            s->set_converge(km.converge);
            s->set_tolerance(gb.tolerance);
            s->set_spatial_order(gb.spatial_order);
            kmeans = [s](size_t a, size_t b, std::shared_ptr<const std::vector<P>> c, std::shared_ptr<std::vector<P>> e,
                         std::shared_ptr<std::vector<M>> f, std::shared_ptr<std::vector<L>> g) {
                return (*s)(a, b, c, e, f, g);
            };
        } else {
            auto s = std::make_shared<KmeansSingleStageBuffered<P, L, M>>();
            BufferedOptions bo;
            bo.device_budget_bytes = (uint64_t)gb.device_budget_mib << 20;
            bo.chunk_bytes = (uint64_t)gb.chunk_mib << 20;
            s->set_options(bo);
            s->set_fused(fu);
            s->set_converge(km.converge);
            s->set_tolerance(gb.tolerance);
            kmeans = [s](size_t a, size_t b, std::shared_ptr<const std::vector<P>> c, std::shared_ptr<std::vector<P>> e,
                         std::shared_ptr<std::vector<M>> f, std::shared_ptr<std::vector<L>> g) {
                return (*s)(a, b, c, e, f, g);
            };
        }
        if (opt.verbose_) std::cout << "Fused device: " << fu.device << std::endl;
    } else {
        throw std::invalid_argument(pipe);
    }

    auto centroids = std::make_shared<std::vector<P>>(k * d);
    auto masses = std::make_shared<std::vector<M>>(k);
    auto labels = std::make_shared<std::vector<L>>(n);
    BenchStats bs;
    bs.num_features = d;
    bs.num_points = n;
    bs.num_clusters = k;
    uint64_t verify_res = 0;
    double mse = 0.0;
    std::vector<P> ref_c(k * d);
    std::vector<M> ref_m(k);
    std::vector<L> ref_l(n);
    if (verify) {
        first_x(*sp, n, d, k, ref_c);
        verify_naive<P, L, M>((uint32_t)km.iterations, *sp, n, d, ref_c, ref_m, ref_l);
        first_x(*sp, n, d, k, *centroids);
        kmeans(km.iterations, d, sp, centroids, masses, labels);
        for (size_t i = 0; i < n; ++i) verify_res += (*labels)[i] != ref_l[i];
        double s = 0, comp = 0;
        for (size_t i = 0; i < k * d; ++i) {
            double x = (double)(*centroids)[i] - (double)ref_c[i];
            double y = x * x - comp, t = s + y;
            comp = (t - s) - y;
            s = t;
        }
        mse = s / (double)(k * d);
    } else {
        for (uint32_t r = 0; r < runs; ++r) {
            first_x(*sp, n, d, k, *centroids);
            auto t0 = std::chrono::steady_clock::now();
            auto m = kmeans(km.iterations, d, sp, centroids, masses, labels);
            auto t1 = std::chrono::steady_clock::now();
            bs.microseconds.push_back((uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count());
            m->set_run((int)r);
            bs.measurements.push_back(m);
        }
    }
    if (opt.verbose_) {
        std::cout << "Pipeline: " << pipe << " Types: " << km.point_type << " " << km.label_type << " "
                  << km.mass_type << std::endl;
        if (verify) {
            std::cout << "Centroid MSE: " << mse << std::endl;
            if (verify_res == 0) std::cout << "Correct labels" << std::endl;
            else std::cout << verify_res << " incorrect labels" << std::endl;
            std::cout << "Cluster Mass" << std::endl;
            for (auto& m : *masses) std::cout << m << " ";
            std::cout << std::endl << "Cluster Mass (Reference)" << std::endl;
            for (auto& m : ref_m) std::cout << m << " ";
            std::cout << std::endl;
        } else {
            bs.print_times(runs);
        }
    } else if (verify) {
        std::cout << "labels_mismatch " << verify_res << " centroid_mse " << mse << std::endl;
    }
    if (!opt.csv_file_.empty() && !verify) bs.to_csv(opt.csv_file_, opt.input_file_);
    return 1;
}

void print_sizes(const char* key, const size_t v[3]) {
    std::cout << key << "=" << v[0] << "," << v[1] << "," << v[2] << "\n";
}

// Prints every field of the parsed configuration structs, one key=value per
// line, in the .conf key names (unset fields show their defaults).
int print_config(const ConfigurationParser& c) {
    auto b = c.get_benchmark_configuration();
    auto k = c.get_kmeans_configuration();
    auto l = c.get_labeling_configuration();
    auto m = c.get_mass_update_configuration();
    auto u = c.get_centroid_update_configuration();
    auto f = c.get_fused_configuration();
    auto g = c.get_gb300_configuration();
    std::cout << "benchmark.runs=" << b.runs << "\nbenchmark.verify=" << b.verify << "\n";
    std::cout << "kmeans.clusters=" << k.clusters << "\nkmeans.pipeline=" << k.pipeline
              << "\nkmeans.iterations=" << k.iterations << "\nkmeans.converge=" << k.converge
              << "\nkmeans.types.point=" << k.point_type << "\nkmeans.types.label=" << k.label_type
              << "\nkmeans.types.mass=" << k.mass_type << "\n";
    std::cout << "kmeans.labeling.platform=" << l.platform << "\nkmeans.labeling.device=" << l.device
              << "\nkmeans.labeling.strategy=" << l.strategy << "\n";
    print_sizes("kmeans.labeling.global_size", l.global_size);
    print_sizes("kmeans.labeling.local_size", l.local_size);
    std::cout << "kmeans.labeling.vector_length=" << l.vector_length
              << "\nkmeans.labeling.unroll_clusters_length=" << l.unroll_clusters_length
              << "\nkmeans.labeling.unroll_features_length=" << l.unroll_features_length << "\n";
    std::cout << "kmeans.mass_update.platform=" << m.platform << "\nkmeans.mass_update.device=" << m.device
              << "\nkmeans.mass_update.strategy=" << m.strategy << "\n";
    print_sizes("kmeans.mass_update.global_size", m.global_size);
    print_sizes("kmeans.mass_update.local_size", m.local_size);
    std::cout << "kmeans.mass_update.vector_length=" << m.vector_length << "\n";
    std::cout << "kmeans.centroid_update.platform=" << u.platform << "\nkmeans.centroid_update.device=" << u.device
              << "\nkmeans.centroid_update.strategy=" << u.strategy << "\n";
    print_sizes("kmeans.centroid_update.global_size", u.global_size);
    print_sizes("kmeans.centroid_update.local_size", u.local_size);
    std::cout << "kmeans.centroid_update.local_features=" << u.local_features
              << "\nkmeans.centroid_update.thread_features=" << u.thread_features
              << "\nkmeans.centroid_update.vector_length=" << u.vector_length << "\n";
    std::cout << "kmeans.fused.platform=" << f.platform << "\nkmeans.fused.device=" << f.device
              << "\nkmeans.fused.strategy=" << f.strategy << "\n";
    print_sizes("kmeans.fused.global_size", f.global_size);
    print_sizes("kmeans.fused.local_size", f.local_size);
    std::cout << "kmeans.fused.vector_length=" << f.vector_length << "\n";
    std::cout << "kmeans.gb300.device_budget_mib=" << g.device_budget_mib << "\nkmeans.gb300.chunk_mib=" << g.chunk_mib
              << "\nkmeans.gb300.copy_streams=" << g.copy_streams << "\nkmeans.gb300.graphs=" << g.graphs
              << "\nkmeans.gb300.tolerance=" << g.tolerance
              << "\nkmeans.gb300.spatial_order=" << (g.spatial_order > 0 ? "on" : (g.spatial_order < 0 ? "off" : "auto"))
              << "\n";
    return 1;
}

int file_info(const std::string& path) {
    BinaryHeader h = BinaryFormat::read_header(path);
    std::cout << "num_features=" << h.num_features << "\nnum_clusters=" << h.num_clusters
              << "\nnum_points=" << h.num_points << "\n";
    return 1;
}

int generate(const CmdOptions& opt) {
    const uint64_t n = opt.gen_points_, d = opt.gen_features_;
    std::vector<float> host(n * d);
    float* dev = nullptr;
    cuda_check(cudaMalloc(&dev, n * d * sizeof(float)), "cudaMalloc");
    int st = ckm_generate_mixture_f32((uint32_t)d, n, opt.gen_blobs_, opt.gen_seed_, -10.f, 10.f, opt.sigma_lo_,
                                      opt.sigma_hi_, 0, dev, n, nullptr);
    if (st != CKM_OK) {
        cudaFree(dev);
        std::cerr << "generate failed: " << ckm_last_error() << std::endl;
        return -1;
    }
    cuda_check(cudaMemcpy(host.data(), dev, n * d * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
    cudaFree(dev);
    BinaryFormat::write(opt.generate_, host.data(), n, d);
    std::cout << "wrote " << opt.generate_ << " (" << n << " points, " << d << " features)" << std::endl;
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        CmdOptions options;
        if (options.parse(argc, argv) < 0) return options.help_ ? 0 : 1;
        if (!options.generate_.empty()) return generate(options) > 0 ? 0 : 1;
        if (options.transfer_) return transfer_bench(options) > 0 ? 0 : 1;
        if (options.info_) return file_info(options.input_file_) > 0 ? 0 : 1;
        ConfigurationParser config;
        config.parse_file(options.config_file_);
        if (options.print_config_) return print_config(config) > 0 ? 0 : 1;
        auto km = config.get_kmeans_configuration();
        if (km.point_type == "double" && km.label_type == "uint64" && km.mass_type == "uint64")
            return run_bench<double, uint64_t, uint64_t>(options, config) > 0 ? 0 : 1;
        if (km.point_type == "float" && km.label_type == "uint32" && km.mass_type == "uint32")
            return run_bench<float, uint32_t, uint32_t>(options, config) > 0 ? 0 : 1;
        throw std::invalid_argument("Invalid type");
    } catch (const std::exception& e) {
        std::cerr << "ckm_bench: " << e.what() << std::endl;
        return 1;
    }
}
