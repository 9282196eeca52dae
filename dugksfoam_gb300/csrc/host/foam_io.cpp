// OpenFOAM ASCII reader/writer (see foam_io.h).
#include "foam_io.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "dugks/dugks.h"

namespace dugks {
namespace {

struct Tok {
    char p = 0;          // punctuation char, or 0 for a word
    std::string s;       // word text
};

bool slurp(const std::string& path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

void tokenize(const std::string& t, std::vector<Tok>& out) {
    size_t i = 0, n = t.size();
    out.clear();
    out.reserve(n / 6);
    while (i < n) {
        char c = t[i];
        if (std::isspace((unsigned char)c)) { ++i; continue; }
        if (c == '/' && i + 1 < n && t[i + 1] == '/') { while (i < n && t[i] != '\n') ++i; continue; }
        if (c == '/' && i + 1 < n && t[i + 1] == '*') {
            i += 2;
            while (i + 1 < n && !(t[i] == '*' && t[i + 1] == '/')) ++i;
            i += 2;
            continue;
        }
        if (c == '(' || c == ')' || c == '{' || c == '}' || c == '[' || c == ']' || c == ';') {
            Tok k; k.p = c; out.push_back(k); ++i; continue;
        }
        if (c == '"') {
            size_t j = i + 1;
            while (j < n && t[j] != '"') ++j;
            Tok k; k.s = t.substr(i + 1, j - i - 1); out.push_back(k);
            i = j + 1;
            continue;
        }
        size_t j = i;
        while (j < n && !std::isspace((unsigned char)t[j]) && t[j] != '(' && t[j] != ')' && t[j] != '{' &&
               t[j] != '}' && t[j] != '[' && t[j] != ']' && t[j] != ';')
            ++j;
        Tok k; k.s = t.substr(i, j - i); out.push_back(k);
        i = j;
    }
}

struct Dict;
struct Entry {
    bool isDict = false;
    std::vector<Tok> toks;
    Dict* dict = nullptr;
};
struct Dict {
    std::vector<std::string> keys;
    std::vector<Entry> vals;
    ~Dict() { for (auto& e : vals) delete e.dict; }
    const Entry* find(const std::string& k) const {
        for (size_t i = 0; i < keys.size(); ++i) if (keys[i] == k) return &vals[i];
        return nullptr;
    }
    const Dict* sub(const std::string& k) const {
        const Entry* e = find(k);
        return (e && e->isDict) ? e->dict : nullptr;
    }
};

// Parse entries until '}' (or end); pos is left after the closing brace.
bool parseDict(const std::vector<Tok>& t, size_t& pos, Dict& d, std::string& err) {
    while (pos < t.size()) {
        if (t[pos].p == '}') { ++pos; return true; }
        if (t[pos].p == ';') { ++pos; continue; }
        if (t[pos].p != 0) { err = "unexpected punctuation in dictionary"; return false; }
        std::string key = t[pos++].s;
        Entry e;
        if (pos < t.size() && t[pos].p == '{') {
            ++pos;
            e.isDict = true;
            e.dict = new Dict();
            if (!parseDict(t, pos, *e.dict, err)) { delete e.dict; return false; }
        } else {
            int depth = 0;
            while (pos < t.size()) {
                char p = t[pos].p;
                if (depth == 0 && p == ';') { ++pos; break; }
                if (p == '(' || p == '[' || p == '{') depth++;
                if (p == ')' || p == ']' || p == '}') depth--;
                e.toks.push_back(t[pos++]);
            }
        }
        d.keys.push_back(key);
        d.vals.push_back(std::move(e));
    }
    return true;
}

bool toNum(const std::string& s, double& v) {
    if (s.empty()) return false;
    char* end = nullptr;
    v = std::strtod(s.c_str(), &end);
    return end && *end == 0;
}

// Skip a leading "FoamFile { ... }" header; check the format is ascii.
bool skipHeader(const std::vector<Tok>& t, size_t& pos, std::string& err) {
    pos = 0;
    if (t.size() >= 2 && t[0].p == 0 && t[0].s == "FoamFile" && t[1].p == '{') {
        pos = 2;
        Dict h;
        if (!parseDict(t, pos, h, err)) return false;
        const Entry* f = h.find("format");
        if (f && !f->toks.empty() && f->toks[0].s != "ascii") { err = "binary OpenFOAM files are not supported"; return false; }
    }
    return true;
}

// A list "N ( items )", "( items )" or "N{value}" of scalars/labels.
bool parseScalarList(const std::vector<Tok>& t, size_t& pos, std::vector<double>& out, std::string& err) {
    out.clear();
    long n = -1;
    double v;
    if (pos < t.size() && t[pos].p == 0 && toNum(t[pos].s, v)) { n = (long)v; ++pos; }
    if (pos < t.size() && t[pos].p == '{') {
        ++pos;
        if (pos >= t.size() || !toNum(t[pos].s, v)) { err = "bad uniform list"; return false; }
        out.assign(n < 0 ? 0 : n, v);
        pos += 2;
        return true;
    }
    if (pos >= t.size() || t[pos].p != '(') { err = "expected '(' in list"; return false; }
    ++pos;
    if (n >= 0) out.reserve(n);
    while (pos < t.size() && t[pos].p != ')') {
        if (!toNum(t[pos].s, v)) { err = "non-numeric list entry '" + t[pos].s + "'"; return false; }
        out.push_back(v);
        ++pos;
    }
    ++pos;
    if (n >= 0 && (long)out.size() != n) { err = "list length mismatch"; return false; }
    return true;
}

bool parseVectorList(const std::vector<Tok>& t, size_t& pos, std::vector<double>& out, std::string& err) {
    out.clear();
    long n = -1;
    double v;
    if (pos < t.size() && t[pos].p == 0 && toNum(t[pos].s, v)) { n = (long)v; ++pos; }
    if (pos < t.size() && t[pos].p == '{') {  // N{(x y z)}
        ++pos;
        double x[3];
        if (t[pos].p != '(') { err = "bad uniform vector list"; return false; }
        for (int k = 0; k < 3; ++k) if (!toNum(t[pos + 1 + k].s, x[k])) { err = "bad vector"; return false; }
        pos += 6;
        for (long i = 0; i < n; ++i) out.insert(out.end(), x, x + 3);
        return true;
    }
    if (pos >= t.size() || t[pos].p != '(') { err = "expected '(' in vector list"; return false; }
    ++pos;
    if (n >= 0) out.reserve(3 * n);
    while (pos < t.size() && t[pos].p != ')') {
        if (t[pos].p != '(' || pos + 4 >= t.size()) { err = "expected '(' for vector"; return false; }
        for (int k = 0; k < 3; ++k) {
            if (!toNum(t[pos + 1 + k].s, v)) { err = "bad vector component"; return false; }
            out.push_back(v);
        }
        if (t[pos + 4].p != ')') { err = "vector with != 3 components"; return false; }
        pos += 5;
    }
    ++pos;
    if (n >= 0 && (long)out.size() != 3 * n) { err = "vector list length mismatch"; return false; }
    return true;
}

bool readListFile(const std::string& path, std::vector<Tok>& t, size_t& pos, std::string& err) {
    std::string txt;
    if (!slurp(path, txt)) { err = "cannot read " + path; return false; }
    tokenize(txt, t);
    if (!skipHeader(t, pos, err)) { err = path + ": " + err; return false; }
    return true;
}

bool readFaces(const std::string& path, FoamCase& c, std::string& err) {
    std::vector<Tok> t;
    size_t pos;
    std::string txt;
    if (!slurp(path, txt)) { err = "cannot read " + path; return false; }
    tokenize(txt, t);
    bool compact = txt.find("faceCompactList") != std::string::npos;
    if (!skipHeader(t, pos, err)) return false;
    c.faceOffsets.clear();
    c.faceVerts.clear();
    if (compact) {
        std::vector<double> off, verts;
        if (!parseScalarList(t, pos, off, err) || !parseScalarList(t, pos, verts, err)) { err = path + ": " + err; return false; }
        for (double x : off) c.faceOffsets.push_back((int32_t)x);
        for (double x : verts) c.faceVerts.push_back((int32_t)x);
        return true;
    }
    double v;
    long n = -1;
    if (pos < t.size() && toNum(t[pos].s, v)) { n = (long)v; ++pos; }
    if (pos >= t.size() || t[pos].p != '(') { err = path + ": expected '('"; return false; }
    ++pos;
    c.faceOffsets.push_back(0);
    while (pos < t.size() && t[pos].p != ')') {
        double m;
        if (!toNum(t[pos].s, m) || pos + 1 >= t.size() || t[pos + 1].p != '(') { err = path + ": bad face"; return false; }
        pos += 2;
        for (long k = 0; k < (long)m; ++k) {
            if (!toNum(t[pos].s, v)) { err = path + ": bad face vertex"; return false; }
            c.faceVerts.push_back((int32_t)v);
            ++pos;
        }
        if (t[pos].p != ')') { err = path + ": face size mismatch"; return false; }
        ++pos;
        c.faceOffsets.push_back((int32_t)c.faceVerts.size());
    }
    if (n >= 0 && (long)c.faceOffsets.size() - 1 != n) { err = path + ": face count mismatch"; return false; }
    return true;
}

bool lastNumber(const Entry* e, double& v) {
    if (!e) return false;
    for (size_t i = e->toks.size(); i-- > 0;)
        if (e->toks[i].p == 0 && toNum(e->toks[i].s, v)) return true;
    return false;
}

// Field value "uniform X", "uniform (x y z)", "nonuniform List<...> N (...)".
bool fieldValues(const Entry* e, int n, int ncmp, std::vector<double>& out, std::string& err) {
    if (!e || e->toks.empty()) { err = "missing value"; return false; }
    const auto& t = e->toks;
    if (t[0].s == "uniform") {
        double x[3] = {0, 0, 0};
        if (ncmp == 1) {
            if (t.size() < 2 || !toNum(t[1].s, x[0])) { err = "bad uniform scalar"; return false; }
        } else {
            if (t.size() < 6 || t[1].p != '(') { err = "bad uniform vector"; return false; }
            for (int k = 0; k < 3; ++k) if (!toNum(t[2 + k].s, x[k])) { err = "bad uniform vector"; return false; }
        }
        out.clear();
        for (int i = 0; i < n; ++i) out.insert(out.end(), x, x + ncmp);
        return true;
    }
    if (t[0].s == "nonuniform") {
        size_t pos = 1;
        if (pos < t.size() && t[pos].s.rfind("List", 0) == 0) ++pos;
        bool ok = ncmp == 1 ? parseScalarList(t, pos, out, err) : parseVectorList(t, pos, out, err);
        if (!ok) return false;
        if ((int)out.size() != n * ncmp) { err = "nonuniform field size mismatch"; return false; }
        return true;
    }
    err = "unsupported field value '" + t[0].s + "'";
    return false;
}

bool readField(const std::string& path, Dict& d, std::string& err) {
    std::string txt;
    if (!slurp(path, txt)) { err = "cannot read " + path; return false; }
    std::vector<Tok> t;
    tokenize(txt, t);
    size_t pos = 0;
    if (!skipHeader(t, pos, err)) return false;
    if (!parseDict(t, pos, d, err)) { err = path + ": " + err; return false; }
    return true;
}

}  // namespace

bool read_foam_case(const std::string& dir, FoamCase& c, std::string& err) {
    const std::string pm = dir + "/constant/polyMesh/";
    std::vector<Tok> t;
    size_t pos;
    std::vector<double> tmp;
    // points
    if (!readListFile(pm + "points", t, pos, err) || !parseVectorList(t, pos, c.points, err)) {
        err = "points: " + err; return false;
    }
    if (!readFaces(pm + "faces", c, err)) return false;
    c.nFaces = (int)c.faceOffsets.size() - 1;
    if (!readListFile(pm + "owner", t, pos, err) || !parseScalarList(t, pos, tmp, err)) { err = "owner: " + err; return false; }
    c.owner.assign(tmp.begin(), tmp.end());
    if (!readListFile(pm + "neighbour", t, pos, err) || !parseScalarList(t, pos, tmp, err)) {
        err = "neighbour: " + err; return false;
    }
    c.neighbour.assign(tmp.begin(), tmp.end());
    c.nInternal = (int)c.neighbour.size();
    if ((int)c.owner.size() != c.nFaces) { err = "owner size != number of faces"; return false; }
    int mx = -1;
    for (int32_t o : c.owner) mx = o > mx ? o : mx;
    for (int32_t o : c.neighbour) mx = o > mx ? o : mx;
    c.nCells = mx + 1;
    // boundary
    if (!readListFile(pm + "boundary", t, pos, err)) return false;
    {
        double v;
        if (pos < t.size() && toNum(t[pos].s, v)) ++pos;
        if (pos >= t.size() || t[pos].p != '(') { err = "boundary: expected '('"; return false; }
        ++pos;
        while (pos < t.size() && t[pos].p != ')') {
            std::string name = t[pos++].s;
            if (pos >= t.size() || t[pos].p != '{') { err = "boundary: expected '{'"; return false; }
            ++pos;
            Dict d;
            if (!parseDict(t, pos, d, err)) return false;
            double nf, sf;
            const Entry* te = d.find("type");
            if (!lastNumber(d.find("nFaces"), nf) || !lastNumber(d.find("startFace"), sf) || !te || te->toks.empty()) {
                err = "boundary: patch " + name + " lacks type/nFaces/startFace";
                return false;
            }
            c.patchNames.push_back(name);
            c.patchTypes.push_back(te->toks[0].s);
            c.patchSize.push_back((int32_t)nf);
            c.patchStart.push_back((int32_t)sf);
        }
    }
    const int nP = (int)c.patchNames.size();
    const int nB = c.nFaces - c.nInternal;
    // fields
    Dict frho, fU, fT;
    if (!readField(dir + "/0/rho", frho, err) || !readField(dir + "/0/U", fU, err) || !readField(dir + "/0/T", fT, err))
        return false;
    if (!fieldValues(frho.find("internalField"), c.nCells, 1, c.rho0, err)) { err = "0/rho internalField: " + err; return false; }
    if (!fieldValues(fU.find("internalField"), c.nCells, 3, c.U0, err)) { err = "0/U internalField: " + err; return false; }
    if (!fieldValues(fT.find("internalField"), c.nCells, 1, c.T0, err)) { err = "0/T internalField: " + err; return false; }
    const Dict* brho = frho.sub("boundaryField");
    const Dict* bU = fU.sub("boundaryField");
    const Dict* bT = fT.sub("boundaryField");
    if (!brho || !bU || !bT) { err = "0/{rho,U,T}: missing boundaryField"; return false; }
    c.wallU.assign(3 * (size_t)nB, 0.0);
    c.wallT.assign(nB, 0.0);
    c.bndRho.assign(nB, 0.0);
    c.patchPressure.assign(nP, 0.0);
    c.patchTzg.assign(nP, 0);
    c.patchUzg.assign(nP, 0);
    c.rhoBC.clear();
    c.patchKind.clear();
    // rho boundary type -> kind (discreteVelocity::setBCtype, discreteVelocity.C:250-300)
    static const std::pair<const char*, int> kKinds[] = {
        {"calculatedMaxwell", DUGKS_PATCH_MAXWELL}, {"empty", DUGKS_PATCH_EMPTY},
        {"zeroGradient", DUGKS_PATCH_ZERO_GRADIENT}, {"fixedValue", DUGKS_PATCH_FIXED_VALUE},
        {"farField", DUGKS_PATCH_FAR_FIELD}, {"pressureIn", DUGKS_PATCH_PRESSURE_IN},
        {"pressureOut", DUGKS_PATCH_PRESSURE_OUT}, {"symmetryMod", DUGKS_PATCH_SYMMETRY_MOD},
        {"symmetryPlane", DUGKS_PATCH_SYMMETRY_PLANE}};
    for (int p = 0; p < nP; ++p) {
        const Dict* pr = brho->sub(c.patchNames[p]);
        const Entry* ty = pr ? pr->find("type") : nullptr;
        // an empty polyMesh patch without a field entry is empty (as OpenFOAM's
        // boundary-field reader fills unlisted empty patches)
        const bool emptyMesh = c.patchTypes[p] == "empty";
        if ((!ty || ty->toks.empty()) && !emptyMesh) {
            err = "0/rho: no boundary entry for patch " + c.patchNames[p];
            return false;
        }
        std::string type = (ty && !ty->toks.empty()) ? ty->toks[0].s : std::string("empty");
        c.rhoBC.push_back(type);
        int kind = -1;
        for (const auto& k : kKinds)
            if (type == k.first) kind = k.second;
        if (kind < 0) {
            err = "unsupported rho boundary type '" + type + "' on patch " + c.patchNames[p] +
                  " (supported: calculatedMaxwell, zeroGradient, fixedValue, farField, pressureIn, pressureOut, "
                  "symmetryMod, symmetryPlane, empty)";
            return false;
        }
        c.patchKind.push_back(kind);
        if (kind == DUGKS_PATCH_EMPTY) continue;
        const int s = c.patchStart[p] - c.nInternal, n = c.patchSize[p];
        if (kind == DUGKS_PATCH_FIXED_VALUE || kind == DUGKS_PATCH_FAR_FIELD) {
            std::vector<double> rv;
            if (!fieldValues(pr->find("value"), n, 1, rv, err)) { err = "0/rho " + c.patchNames[p] + ": " + err; return false; }
            for (int i = 0; i < n; ++i) c.bndRho[s + i] = rv[i];
        }
        if (kind == DUGKS_PATCH_PRESSURE_IN || kind == DUGKS_PATCH_PRESSURE_OUT) {
            const char* key = kind == DUGKS_PATCH_PRESSURE_IN ? "pressureIn" : "pressureOut";
            if (!lastNumber(pr->find(key), c.patchPressure[p])) {
                err = std::string("0/rho ") + c.patchNames[p] + ": missing " + key;
                return false;
            }
        }
        // U and T patch values: the "value" entry, else the owner cells' initial
        // values (zeroGradient-like entries without a value)
        const Dict* pu = bU->sub(c.patchNames[p]);
        const Dict* pt = bT->sub(c.patchNames[p]);
        if (!pu || !pt) { err = "0/U or 0/T: no boundary entry for patch " + c.patchNames[p]; return false; }
        auto isZG = [](const Dict* d) {
            const Entry* t = d->find("type");
            return t && !t->toks.empty() && t->toks[0].s == "zeroGradient";
        };
        c.patchTzg[p] = isZG(pt) ? 1 : 0;
        c.patchUzg[p] = isZG(pu) ? 1 : 0;
        std::vector<double> uv, tv;
        const bool needValues = kind == DUGKS_PATCH_MAXWELL;
        if (pu->find("value") || needValues) {
            if (!fieldValues(pu->find("value"), n, 3, uv, err)) { err = "0/U " + c.patchNames[p] + ": " + err; return false; }
        }
        if (pt->find("value") || needValues) {
            if (!fieldValues(pt->find("value"), n, 1, tv, err)) { err = "0/T " + c.patchNames[p] + ": " + err; return false; }
        }
        for (int i = 0; i < n; ++i) {
            const int own = c.owner[c.patchStart[p] + i];
            for (int k = 0; k < 3; ++k)
                c.wallU[3 * (size_t)(s + i) + k] = uv.empty() ? c.U0[3 * (size_t)own + k] : uv[3 * (size_t)i + k];
            c.wallT[s + i] = tv.empty() ? c.T0[own] : tv[i];
        }
    }
    // DVMProperties
    Dict dvm;
    if (!readField(dir + "/constant/DVMProperties", dvm, err)) return false;
    const Dict* fp = dvm.sub("fvDVMparas");
    const Dict* gp = dvm.sub("gasProperties");
    if (!fp || !gp) { err = "DVMProperties: missing fvDVMparas/gasProperties"; return false; }
    double v;
    if (!lastNumber(fp->find("nDV"), v)) { err = "DVMProperties: nDV"; return false; }
    c.nDV = (int)v;
    if (!lastNumber(fp->find("xiMax"), c.xiMax) || !lastNumber(fp->find("xiMin"), c.xiMin)) {
        err = "DVMProperties: xiMax/xiMin"; return false;
    }
    if (const Entry* mf = fp->find("macroFlux"))
        if (!mf->toks.empty()) c.macroFlux = mf->toks[0].s;
    if (c.macroFlux != "no") { err = "DVMProperties: macroFlux other than \"no\" is not supported"; return false; }
    if (!lastNumber(gp->find("R"), c.R) || !lastNumber(gp->find("omega"), c.omega) || !lastNumber(gp->find("Tref"), c.Tref) ||
        !lastNumber(gp->find("muRef"), c.muRef) || !lastNumber(gp->find("Pr"), c.Pr)) {
        err = "DVMProperties: gasProperties needs R, omega, Tref, muRef, Pr";
        return false;
    }
    c.KInner = lastNumber(gp->find("KInner"), v) ? (int)v : 0;
    // DFwriteCellList (labelList, top level of DVMProperties, fvDVM.C:1067):
    // the labels inside the parentheses (a leading count is not a label)
    c.dfCells.clear();
    if (const Entry* dl = dvm.find("DFwriteCellList")) {
        int depth = 0;
        for (const Tok& t : dl->toks) {
            if (t.p == '(') ++depth;
            else if (t.p == ')') --depth;
            else if (t.p == 0 && depth > 0 && toNum(t.s, v)) c.dfCells.push_back((int32_t)v);
        }
        for (int32_t id : c.dfCells)
            if (id < 0 || id >= c.nCells) { err = "DVMProperties: DFwriteCellList holds a cell out of range"; return false; }
    }
    if (!readListFile(dir + "/constant/Xis", t, pos, err) || !parseScalarList(t, pos, c.xis, err)) { err = "Xis: " + err; return false; }
    if (!readListFile(dir + "/constant/weights", t, pos, err) || !parseScalarList(t, pos, c.weights, err)) {
        err = "weights: " + err; return false;
    }
    if ((int)c.xis.size() != c.nDV || (int)c.weights.size() != c.nDV) {
        err = "Xis/weights length differs from nDV"; return false;
    }
    // controlDict
    Dict cd;
    if (readField(dir + "/system/controlDict", cd, err)) {
        for (size_t i = 0; i < cd.keys.size(); ++i)
            if (!cd.vals[i].isDict && !cd.vals[i].toks.empty()) c.control[cd.keys[i]] = cd.vals[i].toks[0].s;
        lastNumber(cd.find("deltaT"), c.deltaT);
    }
    err.clear();
    return true;
}

namespace {
void header(std::ostream& o, const char* cls, const std::string& obj) {
    o << "FoamFile\n{\n    version     2.0;\n    format      ascii;\n    class       " << cls
      << ";\n    object      " << obj << ";\n}\n\n";
}
}  // namespace

bool write_scalar_list(const std::string& path, const std::string& object, const double* v, int n,
                       std::string& err) {
    std::ofstream o(path);
    if (!o) { err = "cannot write " + path; return false; }
    o.precision(17);
    header(o, "scalarList", object);
    o << n << "\n(\n";
    for (int i = 0; i < n; ++i) o << v[i] << "\n";
    o << ")\n";
    return (bool)o;
}

bool write_vol_field(const std::string& path, const std::string& name, const std::string& dims, int ncomp,
                     const double* internal, int n, const std::vector<PatchOut>& patches, std::string& err) {
    const char* cls = ncomp == 1 ? "volScalarField" : (ncomp == 3 ? "volVectorField" : "volTensorField");
    const char* lst = ncomp == 1 ? "scalar" : (ncomp == 3 ? "vector" : "tensor");
    if (ncomp != 1 && ncomp != 3 && ncomp != 9) { err = "write_vol_field: ncomp must be 1, 3 or 9"; return false; }
    std::ofstream o(path);
    if (!o) { err = "cannot write " + path; return false; }
    o.precision(17);
    auto item = [&](const double* v) {
        if (ncomp == 1) { o << v[0]; return; }
        o << "(";
        for (int k = 0; k < ncomp; ++k) o << (k ? " " : "") << v[k];
        o << ")";
    };
    header(o, cls, name);
    o << "dimensions      " << dims << ";\n\n";
    if (internal) {
        o << "internalField   nonuniform List<" << lst << ">\n" << n << "\n(\n";
        for (int i = 0; i < n; ++i) { item(internal + (size_t)ncomp * i); o << "\n"; }
        o << ")\n;\n\n";
    } else {
        const double zero[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        o << "internalField   uniform ";
        item(zero);
        o << ";\n\n";
    }
    o << "boundaryField\n{\n";
    for (const PatchOut& p : patches) {
        o << "    " << p.name << "\n    {\n        type            " << p.type << ";\n";
        if (!p.extra.empty()) {
            const size_t sp = p.extra.find(' ');
            o << "        " << p.extra.substr(0, sp) << std::string(sp < 16 ? 16 - sp : 1, ' ') << p.extra.substr(sp + 1)
              << ";\n";
        }
        if (p.type != "empty" && p.type != "symmetryPlane") {
            const size_t m = p.values.size() / ncomp;
            o << "        value           nonuniform List<" << lst << "> " << m << "(";
            for (size_t i = 0; i < m; ++i) { o << (i ? " " : ""); item(p.values.data() + ncomp * i); }
            o << ");\n";
        }
        o << "    }\n";
    }
    o << "}\n";
    return (bool)o;
}

}  // namespace dugks
