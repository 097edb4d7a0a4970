// CConfiguration.hpp -- the reference's conf.xml schema (src/CConfiguration.hpp,
// conf.xml) read by a small hand-written parser: the reference's tinyxml2
// dependency is not vendored.  Root `lbm-configuration` with children
//   physics    viscosity, gravitation/{x,y,z}, cavity-velocity/{x,y,z,w}
//   grid       domain-size/{x,y,z}, subdomain-num/{x,y,z},
//              domian-length/{x,y,z}   (the reference's spelling)
//   simulation loops, timestep, visualization/VTK, validate
//   device     kernel-count, device-number
// Optional additions (ignored by the reference, which looks elements up by
// name): physics/lattice/{tau, lid-velocity, reynolds, smagorinsky, storage,
// seed, perturbation}.  When present, tau (or reynolds) and the lid speed
// are taken in lattice units.
#ifndef LBM_GB300_CCONFIGURATION_HPP
#define LBM_GB300_CCONFIGURATION_HPP

#include <cstdlib>
#include <fstream>
#include <iostream>
#include <list>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "CVector.hpp"

namespace lbmxml {
struct Node {
    std::string name, text;
    std::vector<std::unique_ptr<Node>> kids;
    const Node *child(const std::string &n) const {
        for (auto &k : kids)
            if (k->name == n) return k.get();
        return nullptr;
    }
};

// Elements, text, comments, <?...?> and <!...> declarations; no attributes
// are needed by the schema (they are skipped).
inline std::unique_ptr<Node> parse(const std::string &s, std::string &err) {
    auto root = std::make_unique<Node>();
    std::vector<Node *> st{root.get()};
    size_t i = 0;
    while (i < s.size()) {
        if (s[i] != '<') {
            size_t j = s.find('<', i);
            if (j == std::string::npos) j = s.size();
            st.back()->text += s.substr(i, j - i);
            i = j;
            continue;
        }
        if (s.compare(i, 4, "<!--") == 0) {
            size_t j = s.find("-->", i);
            if (j == std::string::npos) { err = "unterminated comment"; return nullptr; }
            i = j + 3;
            continue;
        }
        if (s.compare(i, 2, "<?") == 0 || s.compare(i, 2, "<!") == 0) {
            size_t j = s.find('>', i);
            if (j == std::string::npos) { err = "unterminated declaration"; return nullptr; }
            i = j + 1;
            continue;
        }
        size_t j = s.find('>', i);
        if (j == std::string::npos) { err = "unterminated tag"; return nullptr; }
        std::string tag = s.substr(i + 1, j - i - 1);
        i = j + 1;
        if (!tag.empty() && tag[0] == '/') {
            std::string n = tag.substr(1);
            while (!n.empty() && isspace((unsigned char)n.back())) n.pop_back();
            if (st.size() < 2 || st.back()->name != n) { err = "mismatched </" + n + ">"; return nullptr; }
            st.pop_back();
            continue;
        }
        bool self_close = !tag.empty() && tag.back() == '/';
        if (self_close) tag.pop_back();
        size_t sp = tag.find_first_of(" \t\r\n");
        auto node = std::make_unique<Node>();
        node->name = tag.substr(0, sp);
        Node *raw = node.get();
        st.back()->kids.push_back(std::move(node));
        if (!self_close) st.push_back(raw);
    }
    if (st.size() != 1) { err = "unclosed element <" + st.back()->name + ">"; return nullptr; }
    return root;
}
}  // namespace lbmxml

template <typename T>
class CConfiguration {
public:
    CVector<3, int> domain_size{32, 32, 32};
    CVector<3, int> subdomain_num{1, 1, 1};
    CVector<3, T> domain_length{T(0.1), T(0.1), T(0.1)};
    CVector<3, T> gravitation{T(0), T(-9.81), T(0)};
    T viscosity = T(0.001308);
    CVector<4, T> drivenCavityVelocity{T(100), T(0), T(0), T(1)};
    size_t computation_kernel_count = 128;
    int device_nr = 0;
    bool do_visualization = false;
    T timestep = T(-1);
    int loops = -1;
    bool do_validate = false;
    std::list<int> lbm_opencl_number_of_registers_list;
    std::list<int> lbm_opencl_number_of_threads_list;
    bool debug_mode = false;
    // append the timing of each run to output/benchmark/benchmark_<subdomains>.ini
    // (the reference's BENCHMARK build, src/CController.hpp:445-477); a build with
    // -DBENCHMARK=1 turns it on by default, the command line with -b
#if defined(BENCHMARK) && BENCHMARK
    bool benchmark = true;
#else
    bool benchmark = false;
#endif

    // optional lattice-unit additions
    bool lattice_units = false;
    T lattice_tau = T(0);
    T lattice_reynolds = T(0);
    T lattice_lid = T(0);
    T smagorinsky = T(0);
    std::string storage = "";
    unsigned long long seed = 0;
    T perturbation = T(0);

    CConfiguration() {}
    explicit CConfiguration(const std::string &file) { loadFile(file); }

    void loadFile(const std::string &file_name) {
        std::ifstream f(file_name);
        if (!f) throw "Loading XML file failed";
        std::stringstream ss;
        ss << f.rdbuf();
        std::string err;
        auto doc = lbmxml::parse(ss.str(), err);
        if (!doc) throw "Loading XML file failed";
        const lbmxml::Node *root = doc->child("lbm-configuration");
        if (!root) throw "Loading XML file failed: no <lbm-configuration>";
        interpret(root);
    }

    void printMe() const {
        std::cout << "################\n# CONFIGURATION \n################\n"
                  << "PHYSICS: \n\t    VISCOSITY: " << viscosity << "\n\t  GRAVITATION: " << gravitation
                  << "\n     CAVITY VEL: " << drivenCavityVelocity << "\nGRID: \n\t  DOMAIN_SIZE: " << domain_size
                  << "\n\tSUBDOMIAN_NUM: " << subdomain_num << "\nSIMULATION: \n\t        LOOPS: " << loops
                  << "\n\t     TIMESTEP: " << timestep << "\n\t          VTK: " << do_visualization
                  << "\n\t     VALIDATE: " << do_validate << "\nDEVICE: \n  KERNEL_COUNT: "
                  << computation_kernel_count << "\n\t    DEVICE_NR: " << device_nr << std::endl;
    }

private:
    static const lbmxml::Node *req(const lbmxml::Node *n, const char *name) {
        const lbmxml::Node *c = n ? n->child(name) : nullptr;
        if (!c) {
            static std::string msg;
            msg = std::string("conf.xml: missing element <") + name + ">";
            throw msg.c_str();
        }
        return c;
    }
    static double num(const lbmxml::Node *n, const char *name) { return atof(req(n, name)->text.c_str()); }
    template <int D, typename V>
    static void vec(const lbmxml::Node *n, const char *name, CVector<D, V> &v) {
        static const char *ax[4] = {"x", "y", "z", "w"};
        const lbmxml::Node *c = req(n, name);
        for (int a = 0; a < D; a++) v[a] = (V)num(c, ax[a]);
    }

    void interpret(const lbmxml::Node *root) {
        const lbmxml::Node *dev = req(root, "device");
        computation_kernel_count = (size_t)num(dev, "kernel-count");
        device_nr = (int)num(dev, "device-number");
        const lbmxml::Node *grid = req(root, "grid");
        vec(grid, "domain-size", domain_size);
        vec(grid, "subdomain-num", subdomain_num);
        vec(grid, "domian-length", domain_length);
        const lbmxml::Node *phy = req(root, "physics");
        viscosity = (T)num(phy, "viscosity");
        vec(phy, "gravitation", gravitation);
        vec(phy, "cavity-velocity", drivenCavityVelocity);
        const lbmxml::Node *sim = req(root, "simulation");
        loops = (int)num(sim, "loops");
        timestep = (T)num(sim, "timestep");
        do_visualization = num(req(sim, "visualization"), "VTK") != 0;
        do_validate = num(sim, "validate") != 0;
        if (const lbmxml::Node *lat = phy->child("lattice")) {
            lattice_units = true;
            if (lat->child("tau")) lattice_tau = (T)num(lat, "tau");
            if (lat->child("reynolds")) lattice_reynolds = (T)num(lat, "reynolds");
            lattice_lid = (T)num(lat, "lid-velocity");
            if (lat->child("smagorinsky")) smagorinsky = (T)num(lat, "smagorinsky");
            if (lat->child("storage")) {
                storage = lat->child("storage")->text;
                while (!storage.empty() && isspace((unsigned char)storage.back())) storage.pop_back();
                while (!storage.empty() && isspace((unsigned char)storage.front())) storage.erase(0, 1);
            }
            if (lat->child("seed")) seed = (unsigned long long)num(lat, "seed");
            if (lat->child("perturbation")) perturbation = (T)num(lat, "perturbation");
            if (!(lattice_tau > T(0)) && !(lattice_reynolds > T(0)))
                throw "conf.xml: <lattice> needs <tau> or <reynolds>";
        }
    }
};

template <class C>
class Singleton {
public:
    static C *Instance() {
        static C instance;
        return &instance;
    }
};

#endif
