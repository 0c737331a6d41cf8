// simplic_solveVofEqu.hpp -- C++ host facade over the simplic C ABI.
//
// Mirrors Foam::geometricVofExt::SimPLIC::solveVofEqu
// (src/SimPLIC/solveVofEqu/solveVofEqu.H:67-216): built from the volume
// fraction, face flux and velocity fields (held by reference and read on
// every call), configured from the solvers."alpha.*" entry of fvSolution
// (solveVofEqu.C:68), with reconstruct(), advect(Sp, Su), getRhoPhi(),
// alphaPhi() and the three timers.  Fields are plain contiguous arrays in
// OpenFOAM order; an OpenFOAM adapter passes primitiveField() data.
// Errors throw simplic::Error (the reference aborts with FatalError).
#pragma once

#include <cctype>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "simplic.h"
#include "simplic_mlp.h"

namespace simplic {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int r, const simplic_handle* h) {
    if (r != SIMPLIC_OK) throw Error(r, simplic_last_error(h));
}

// ---------------------------------------------------------------------------
// Minimal OpenFOAM dictionary: nested blocks of `key value;` entries,
// comments, quoted regular-expression keys.
// ---------------------------------------------------------------------------
class Dictionary {
public:
    std::map<std::string, std::string> values;
    std::map<std::string, std::shared_ptr<Dictionary>> dicts;
    std::vector<std::string> order;  // insertion order of block keys

    static Dictionary parse(const std::string& text) {
        std::vector<std::string> toks = tokenize(text);
        size_t pos = 0;
        Dictionary d;
        d.parseBlock(toks, pos);
        return d;
    }
    static Dictionary read(const std::string& path) {
        std::ifstream in(path);
        if (!in) throw Error(SIMPLIC_ERR_INVALID_ARGUMENT, "cannot open " + path);
        std::stringstream ss;
        ss << in.rdbuf();
        return parse(ss.str());
    }
    const Dictionary& subDict(const std::string& k) const {
        auto it = dicts.find(k);
        if (it == dicts.end()) throw Error(SIMPLIC_ERR_INVALID_ARGUMENT, "no sub-dictionary " + k);
        return *it->second;
    }
    // mesh.solverDict(name): exact key, else the last matching regex key
    const Dictionary& solverDict(const std::string& field) const {
        const Dictionary& s = dicts.count("solvers") ? subDict("solvers") : *this;
        auto it = s.dicts.find(field);
        if (it != s.dicts.end()) return *it->second;
        for (auto k = s.order.rbegin(); k != s.order.rend(); ++k) {
            if (k->size() >= 2 && (*k)[0] == '"') {
                const std::string pat = k->substr(1, k->size() - 2);
                if (std::regex_match(field, std::regex(pat))) return *s.dicts.at(*k);
            }
        }
        throw Error(SIMPLIC_ERR_INVALID_ARGUMENT, "no solver entry for " + field);
    }
    double getOrDefault(const std::string& k, double def) const {
        auto it = values.find(k);
        return it == values.end() ? def : std::stod(it->second);
    }
    bool getOrDefaultBool(const std::string& k, bool def) const {
        auto it = values.find(k);
        if (it == values.end()) return def;
        std::string v = it->second;
        for (auto& ch : v) ch = char(std::tolower(ch));
        if (v == "true" || v == "on" || v == "yes" || v == "1") return true;
        if (v == "false" || v == "off" || v == "no" || v == "none" || v == "0") return false;
        throw Error(SIMPLIC_ERR_INVALID_ARGUMENT, "bad switch value for " + k);
    }
    std::string getOrDefaultWord(const std::string& k, const std::string& def) const {
        auto it = values.find(k);
        return it == values.end() ? def : it->second;
    }

private:
    static std::vector<std::string> tokenize(const std::string& src) {
        std::string t;
        for (size_t i = 0; i < src.size(); ++i) {  // strip comments
            if (src[i] == '/' && i + 1 < src.size() && src[i + 1] == '/') {
                while (i < src.size() && src[i] != '\n') ++i;
            } else if (src[i] == '/' && i + 1 < src.size() && src[i + 1] == '*') {
                i += 2;
                while (i + 1 < src.size() && !(src[i] == '*' && src[i + 1] == '/')) ++i;
                ++i;
            } else {
                t += src[i];
            }
        }
        std::vector<std::string> out;
        for (size_t i = 0; i < t.size();) {
            const char c = t[i];
            if (std::isspace((unsigned char)c)) {
                ++i;
            } else if (c == '{' || c == '}' || c == ';' || c == '(' || c == ')') {
                out.emplace_back(1, c);
                ++i;
            } else if (c == '"') {
                size_t j = t.find('"', i + 1);
                if (j == std::string::npos) j = t.size() - 1;
                out.push_back(t.substr(i, j - i + 1));
                i = j + 1;
            } else {
                size_t j = i;
                while (j < t.size() && !std::isspace((unsigned char)t[j]) && t[j] != '{' && t[j] != '}' &&
                       t[j] != ';' && t[j] != '(' && t[j] != ')')
                    ++j;
                out.push_back(t.substr(i, j - i));
                i = j;
            }
        }
        return out;
    }
    void parseBlock(const std::vector<std::string>& toks, size_t& pos) {
        while (pos < toks.size()) {
            const std::string key = toks[pos++];
            if (key == "}") return;
            if (pos < toks.size() && toks[pos] == "{") {
                ++pos;
                auto d = std::make_shared<Dictionary>();
                d->parseBlock(toks, pos);
                dicts[key] = d;
                order.push_back(key);
                continue;
            }
            std::string val;
            int depth = 0;
            while (pos < toks.size() && !(toks[pos] == ";" && depth == 0)) {
                if (toks[pos] == "(") ++depth;
                if (toks[pos] == ")") --depth;
                if (!val.empty()) val += ' ';
                val += toks[pos++];
            }
            ++pos;
            values[key] = val;
        }
    }
};

// The dictionary lookups of reconstruction.C:502-516 and advection.C:455-457.
inline simplic_controls controlsFromDict(const Dictionary& d) {
    simplic_controls c;
    simplic_default_controls(&c);
    c.mixed_cell_tol = d.getOrDefault("mixedCellTol", 1e-8);
    c.write_plic_fields = d.getOrDefaultBool("writePlicFields", false);
    c.split_warped_face = d.getOrDefaultBool("splitWarpedFace", false);
    const std::string om = d.getOrDefaultWord("orientationMethod", "isoAlphaGrad");
    if (om == "isoAlphaGrad" || om == "LS")
        c.orientation_method = SIMPLIC_ORIENTATION_ISO_ALPHA_GRAD;
    else if (om == "alphaGrad")
        c.orientation_method = SIMPLIC_ORIENTATION_ALPHA_GRAD;
    else if (om == "isoRDF" || om == "RDF")
        c.orientation_method = SIMPLIC_ORIENTATION_ISO_RDF;
    else
        throw Error(SIMPLIC_ERR_INVALID_ARGUMENT, "Orientation vector calculation method '" + om + "' is not valid");
    c.map_alpha_field = d.getOrDefaultBool("mapAlphaField", false);
    c.iso_rdf_tol = d.getOrDefault("tol", 1e-6);
    c.iso_rdf_rel_tol = d.getOrDefault("relTol", 0.1);
    c.iso_rdf_iterations = int(d.getOrDefault("iterations", 5));
    c.n_alpha_bounds = int(d.getOrDefault("nAlphaBounds", 10));
    c.snap_tol = d.getOrDefault("snapTol", 0.0);
    c.clip = d.getOrDefaultBool("clip", true);
    // the form of the step (no counterpart in the reference): plain FP64
    // (the drop-in), mixed precision, or learned normals (setNetwork)
    const std::string prec = d.getOrDefaultWord("precision", "plain");
    if (prec == "plain")
        c.precision = SIMPLIC_PRECISION_PLAIN_FP64;
    else if (prec == "mixed")
        c.precision = SIMPLIC_PRECISION_MIXED;
    else if (prec == "learned")
        c.precision = SIMPLIC_PRECISION_LEARNED;
    else
        throw Error(SIMPLIC_ERR_INVALID_ARGUMENT, "precision '" + prec + "' is not plain, mixed or learned");
    return c;
}

// ---------------------------------------------------------------------------
// solveVofEqu
// ---------------------------------------------------------------------------
class solveVofEqu {
public:
    static constexpr const char* typeName = "solveVofEqu";

    // alpha1 [nCells] (modified in place by advect), phi [nFaces],
    // U [3 nCells]; Ub [3 nBoundaryFaces] or null (zero gradient).
    solveVofEqu(const simplic_mesh_desc& mesh, std::vector<double>& alpha1, const std::vector<double>& phi,
                const std::vector<double>& U, const Dictionary& solverDict, const std::vector<double>* Ub = nullptr,
                void* cudaStream = nullptr)
        : mesh_(mesh), alpha1_(alpha1), phi_(phi), U_(U), Ub_(Ub), dict_(solverDict),
          ctrl_(controlsFromDict(solverDict)) {
        simplic_handle* h = nullptr;
        check(simplic_create(&mesh, &ctrl_, cudaStream, &h), nullptr);
        h_.reset(h);
    }

    // solveVofEqu.C:96-99
    void reconstruct() { check(simplic_reconstruct(h_.get(), alpha1_.data()), h_.get()); }

    // solveVofEquTemplates.C:35-43 with zeroField sources
    void advect() { advectImpl(nullptr, nullptr); }
    // ... with volScalarField::Internal sources (phase change)
    void advect(const std::vector<double>& Sp, const std::vector<double>& Su) { advectImpl(Sp.data(), Su.data()); }

    // solveVofEqu.C:102-105 -> reconstruction.C:725-784: a static mesh has
    // nothing to map (the reference returns unless the mesh is a
    // dynamicRefineFvMesh that changed)
    void mapAlphaField() {}
    // ... after a refinement, on a solver built for the new mesh: normal
    // [3 nCells] and distance [nCells] are interfaceN / interfaceD mapped
    // onto it (children carry their parent's plane); lower / upper are the
    // dynamicMeshDict lowerRefineLevel / upperRefineLevel
    void mapAlphaField(const std::vector<double>& normal, const std::vector<double>& distance, double lower,
                       double upper) {
        if (!ctrl_.map_alpha_field) return;
        check(simplic_map_alpha_field(h_.get(), alpha1_.data(), normal.data(), distance.data(), lower, upper,
                                      SIMPLIC_MEM_HOST),
              h_.get());
    }
    // reconstruction::interface (reconstruction.C:787-835): the PLIC polygons
    // of the last reconstruct (offsets [n+1], xyz points, cell of each)
    void interface(std::vector<int32_t>& offsets, std::vector<double>& points, std::vector<int32_t>& cells) {
        int32_t nq = 0, np = 0;
        check(simplic_get_interface_polygons(h_.get(), &nq, &np, nullptr, nullptr, nullptr), h_.get());
        offsets.resize(size_t(nq) + 1);
        points.resize(3 * size_t(np));
        cells.resize(size_t(nq));
        check(simplic_get_interface_polygons(h_.get(), &nq, &np, offsets.data(), points.data(), cells.data()),
              h_.get());
    }

    void setDeltaT(double dt) { dt_ = dt; }
    // network of precision "learned": W [4][128][128], b [4][128] (FP32);
    // gateTol is the fallback threshold on the local volume residual
    void setNetwork(const float* W, const float* b, float gateTol = 0.01f) {
        check(simplic_set_network(h_.get(), W, b, gateTol), h_.get());
    }
    void setOldTime(const std::vector<double>* alphaOld) { alphaOld_ = alphaOld; }

    const std::vector<double>& alpha() const { return alpha1_; }
    const Dictionary& dict() const { return dict_; }

    // advection.H:329-343 with dimensioned densities
    std::vector<double> getRhoPhi(double rho1, double rho2) const {
        std::vector<double> out(phi_.size());
        check(simplic_get_rho_phi(h_.get(), rho1, rho2, phi_.data(), out.data(), SIMPLIC_MEM_HOST), h_.get());
        return out;
    }
    const std::vector<double>& alphaPhi() {
        alphaPhi_.resize(phi_.size());
        check(simplic_get_alpha_phi(h_.get(), alphaPhi_.data(), SIMPLIC_MEM_HOST), h_.get());
        return alphaPhi_;
    }
    std::vector<int32_t> mixedCells() const {
        int32_t n = 0;
        check(simplic_get_mixed_cells(h_.get(), &n, nullptr, nullptr), h_.get());
        std::vector<int32_t> c(n);
        check(simplic_get_mixed_cells(h_.get(), &n, c.data(), nullptr), h_.get());
        return c;
    }
    double reconstructionTime() const { return timer(0); }
    double advectionTime() const { return timer(1); }
    double alphaMappingTime() const { return timer(2); }
    simplic_handle* handle() const { return h_.get(); }

private:
    struct Deleter {
        void operator()(simplic_handle* h) const { simplic_destroy(h); }
    };
    void advectImpl(const double* Sp, const double* Su) {
        if (!(dt_ > 0.0)) throw Error(SIMPLIC_ERR_STATE, "setDeltaT before advect");
        simplic_step_inputs in{};
        in.phi = phi_.data();
        in.U = U_.data();
        in.U_boundary = Ub_ ? Ub_->data() : nullptr;
        in.Sp = Sp;
        in.Su = Su;
        in.dt = dt_;
        check(simplic_advect(h_.get(), alpha1_.data(), alphaOld_ ? alphaOld_->data() : nullptr, &in), h_.get());
    }
    double timer(int i) const {
        double t[3] = {0, 0, 0};
        check(simplic_timers(h_.get(), &t[0], &t[1], &t[2]), h_.get());
        return t[i];
    }

    simplic_mesh_desc mesh_;
    std::vector<double>& alpha1_;
    const std::vector<double>& phi_;
    const std::vector<double>& U_;
    const std::vector<double>* Ub_;
    const std::vector<double>* alphaOld_ = nullptr;
    Dictionary dict_;
    simplic_controls ctrl_;
    double dt_ = 0.0;
    std::vector<double> alphaPhi_;
    std::unique_ptr<simplic_handle, Deleter> h_;
};

}  // namespace simplic
