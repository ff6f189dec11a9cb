// JSON input -> Inputs. Each block cites the lines of chiML's
// INPUTS/parallelInputs.cpp whose conversions it keeps.
#include <algorithm>
#include <cmath>
#include <numeric>

#include "model.hpp"

namespace chiml {

const double kSpeedOfLight = 2.9979245e8;
const double kEps0 = 1 / (4 * M_PI * 1.0e-7 * std::pow(kSpeedOfLight, 2.0));
const double kElementaryCharge = 1.6021766208000000926392586608069679194921272585907390121132132243531032145256176590919494628906250000e-19;
const double kHbar = 1.0545718001391127086220667148574871851002905804237980726847871017460777904741746884127674612624536721e-34;

int Inputs::nSteps() const { return static_cast<int>(std::ceil(tMax / dt)); }

namespace {

int find_pt(double pt, double d) { return static_cast<int>(std::floor(pt / d + 0.5)); }

Pol string2pol(const std::string& p) {
    if (p == "Ex") return Pol::EX;
    if (p == "Ey") return Pol::EY;
    if (p == "Ez") return Pol::EZ;
    if (p == "Hx") return Pol::HX;
    if (p == "Hy") return Pol::HY;
    if (p == "Hz") return Pol::HZ;
    if (p == "L") return Pol::L;
    if (p == "R") return Pol::R;
    throw InputError("POLARIZATION undefined");
}

PulseShape string2prof(const std::string& p) {
    if (p == "gaussian") return PulseShape::GAUSSIAN;
    if (p == "BH") return PulseShape::BH;
    if (p == "rectangle") return PulseShape::RECT;
    if (p == "continuous") return PulseShape::CONTINUOUS;
    if (p == "ricker") return PulseShape::RICKER;
    if (p == "ramped_cont") return PulseShape::RAMP_CONT;
    throw InputError("Pulse shape undefined");
}

DtcType string2out(const std::string& t) {
    static const char* names[] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz", "Dx", "Dy", "Dz",
                                  "Bx", "By", "Bz", "E_pow", "H_pow", "Px", "Py", "Pz"};
    for (int i = 0; i < 17; ++i)
        if (t == names[i]) return static_cast<DtcType>(i);
    if (t == "Mx" || t == "My" || t == "Mz" || t.rfind("Chi", 0) == 0)
        throw UnsupportedError("detector type " + t + " needs magnetic or chiral media, which are not supported");
    throw InputError("DTCTYPE (DetectorList.type) from input file not defined");
}

DipOr string2dipor(const std::string& s) {
    if (s == "isotropic") return DipOr::ISOTROPIC;
    if (s == "normal" || s == "tangent" || s == "rel_norm") return DipOr::REL_TO_NORM;
    if (s == "lat_tangent") return DipOr::LAT_TAN;
    if (s == "long_tangent") return DipOr::LONG_TAN;
    if (s == "unidirectional") return DipOr::UNIDIRECTIONAL;
    throw InputError("The dipole orientation style is undefined");
}

// Pulse parameter lists, parallelInputs.cpp:133-172 (sources) and 351-390 (TFSF).
PulseSpec read_pulse(const JNode& pul, double a, double I0) {
    PulseSpec p;
    p.shape = string2prof(pul.get<std::string>("profile"));
    double emax = pul.get<double>("Field_Intensity", 1.0) * a * kEps0 * kSpeedOfLight / I0;
    std::vector<cplx>& f = p.param;
    switch (p.shape) {
        case PulseShape::GAUSSIAN:
            f.push_back(cplx(0.0, -1.0 * pul.get<double>("fcen") * 2 * M_PI));
            f.push_back(1.0 / pul.get<double>("fwidth"));
            f.push_back(pul.get<double>("cutoff") * f[1]);
            f.push_back(pul.get<double>("t_0", std::real(f[1] * f[2])));
            f[2] += f[3];
            break;
        case PulseShape::BH:
            f.push_back(cplx(0.0, -1.0 * pul.get<double>("fcen") * 2 * M_PI));
            f.push_back(pul.get<double>("tau", 1.0 / pul.get<double>("fwidth")));
            // f[2] is read before it exists in the reference (parallelInputs.cpp:145); it is required here
            f.push_back(pul.get<double>("t_0"));
            f.push_back(pul.get<double>("BH1", 0.35875));
            f.push_back(pul.get<double>("BH2", 0.48829));
            f.push_back(pul.get<double>("BH3", 0.14128));
            f.push_back(pul.get<double>("BH4", 0.01168));
            break;
        case PulseShape::RECT:
            f.push_back(pul.get<double>("tau"));
            f.push_back(pul.get<double>("t_0"));
            f.push_back(pul.get<double>("n", 30.0) * 2.0);
            f.push_back(cplx(0.0, -1.0 * pul.get<double>("fcen") * 2 * M_PI));
            break;
        case PulseShape::CONTINUOUS:
            f.push_back(cplx(0.0, -1.0 * pul.get<double>("fcen") * 2 * M_PI));
            break;
        case PulseShape::RAMP_CONT:
            f.push_back(cplx(0.0, -1.0 * pul.get<double>("fcen") * 2 * M_PI));
            f.push_back(pul.get<double>("ramp_val"));
            break;
        case PulseShape::RICKER:
            f.push_back(cplx(0.0, -1.0 * pul.get<double>("fcen") * 2 * M_PI));
            f.push_back(pul.get<double>("fwidth"));
            f.push_back(pul.get<double>("cutoff"));
            break;
    }
    // The amplitude is appended when the source is built (parallelFDTDField.cpp:476)
    f.push_back(emax);
    return p;
}

// Inverse of an n x n column-major matrix in place by LU with partial pivoting
// (LAPACK dgetrf + dgetri semantics, unblocked: the same operation order as the
// one-process reference build). Returns the determinant of the factors as
// UTIL/utilityFxns.hpp:108-116 (getLUFactMatDet) forms it.
double lu_invert(int n, double* a) {
    std::vector<int> ipiv(static_cast<std::size_t>(n));
    for (int j = 0; j < n; ++j) {
        int p = j;
        for (int i = j + 1; i < n; ++i)
            if (std::abs(a[i + j * n]) > std::abs(a[p + j * n])) p = i;
        ipiv[static_cast<std::size_t>(j)] = p + 1;
        if (a[p + j * n] == 0.0) continue;
        if (p != j)
            for (int k = 0; k < n; ++k) std::swap(a[j + k * n], a[p + k * n]);
        for (int i = j + 1; i < n; ++i) a[i + j * n] /= a[j + j * n];
        for (int k = j + 1; k < n; ++k)
            for (int i = j + 1; i < n; ++i) a[i + k * n] -= a[i + j * n] * a[j + k * n];
    }
    double det = 1.0;
    for (int jj = 1; jj <= n; ++jj)
        det *= (ipiv[static_cast<std::size_t>(jj - 1)] != jj) ? -1.0 * a[(jj - 1) * (n + 1)] : a[(jj - 1) * (n + 1)];
    if (det == 0.0) return det;
    std::vector<double> inv(static_cast<std::size_t>(n) * n, 0.0), e(static_cast<std::size_t>(n));
    for (int col = 0; col < n; ++col) {
        std::fill(e.begin(), e.end(), 0.0);
        e[static_cast<std::size_t>(col)] = 1.0;
        for (int i = 0; i < n; ++i) std::swap(e[static_cast<std::size_t>(i)], e[static_cast<std::size_t>(ipiv[static_cast<std::size_t>(i)] - 1)]);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < i; ++k) e[static_cast<std::size_t>(i)] -= a[i + k * n] * e[static_cast<std::size_t>(k)];
        for (int i = n - 1; i >= 0; --i) {
            for (int k = i + 1; k < n; ++k) e[static_cast<std::size_t>(i)] -= a[i + k * n] * e[static_cast<std::size_t>(k)];
            e[static_cast<std::size_t>(i)] /= a[i + i * n];
        }
        for (int i = 0; i < n; ++i) inv[static_cast<std::size_t>(i + col * n)] = e[static_cast<std::size_t>(i)];
    }
    std::copy(inv.begin(), inv.end(), a);
    return det;
}

// Object-space coordinates of p, t_i = sum_k coord[i][k] (p - loc)_k (Obj::RealSpace2ObjectSpace).
std::array<double, 3> to_object(const Object& o, const std::array<double, 3>& p) {
    std::array<double, 3> c = {p[0] - o.loc[0], p[1] - o.loc[1], p[2] - o.loc[2]};
    std::array<double, 3> t;
    for (int i = 0; i < 3; ++i) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += o.coord[i * 3 + k] * c[k];
        t[i] = s;
    }
    return t;
}

// Triangular prism from its three 2-D vertices (Obj.cpp:147-200): the vertices are moved
// to their centroid, which is added to the location, and the vertex matrix rows
// (x, y, 1) are inverted for the barycentric test.
void setup_prism(Object& o, const std::array<std::array<double, 2>, 3>& v) {
    std::array<double, 3> cen = {0.0, 0.0, 0.0};
    for (int ii = 0; ii < 3; ++ii)
        for (int k = 0; k < 2; ++k) cen[k] = cen[k] + v[ii][k] / 3.0;
    for (int k = 0; k < 3; ++k) o.loc[k] = o.loc[k] + cen[k];
    double m[9];
    for (int k = 0; k < 9; ++k) m[k] = 1.0;
    for (int ii = 0; ii < 3; ++ii) {
        o.verts[ii] = {v[ii][0] - cen[0], v[ii][1] - cen[1], 0.0};
        m[ii] = o.verts[ii][0];
        m[ii + 3] = o.verts[ii][1];
    }
    if (lu_invert(3, m) == 0.0) throw InputError("The triangular base is a line.");
    std::copy(m, m + 9, o.invVert.begin());
}

// Tetrahedron from four real-space vertices (Obj.cpp:215-272): rows (x, y, z, 1) inverted.
void setup_tetrahedron(Object& o) {
    double m[16];
    for (int k = 0; k < 16; ++k) m[k] = 1.0;
    for (int ii = 0; ii < 4; ++ii)
        for (int k = 0; k < 3; ++k) m[ii + 4 * k] = o.verts[ii][k];
    if (lu_invert(4, m) == 0.0) throw InputError("The tetrahedron is planer.");
    std::copy(m, m + 16, o.invVert.begin());
}

// Barycentric coordinates of the point (p, 1) with respect to the inverted vertex
// matrix (UTIL/utilityFxns.hpp:130-141, cart2bary): lambda_i = sum_j inv[i n + j] p_j.
template <int N>
std::array<double, N> to_bary(const std::array<double, 16>& inv, const double* p) {
    std::array<double, N> pad;
    for (int j = 0; j < N - 1; ++j) pad[j] = p[j];
    pad[N - 1] = 1.0;
    std::array<double, N> b;
    for (int i = 0; i < N; ++i) {
        double t = 0.0;
        for (int j = 0; j < N; ++j) t += inv[static_cast<std::size_t>(i * N + j)] * pad[j];
        b[i] = t;
    }
    return b;
}

Object make_vacuum_block(const std::array<double, 3>& size) {
    Object o;
    o.shape = Shape::BLOCK;
    o.geo = {size[0], size[1], size[2]};
    o.geoML = o.geo;
    return o;
}


// Named materials (getMater, parallelInputs.cpp:1066-1179). The Lorentz-Drude parameter
// sets are the published ones the reference tabulates (UTIL/dielectric_params.hpp): the
// Rakic et al. sets (Appl. Opt. 37, 5271 (1998)) as {omega_p, then (f, Gamma, omega) per
// oscillator, omega = 0 for the Drude term}, all in eV; the "JM" sets in the same layout
// with the oscillator strength given directly; two quantum-dot resonances. eps_inf is the
// reference's, including the 1 + k 1e-14 of the metals (which keeps them from counting as
// vacuum). The numbers have to be the reference's: they are the material constants.
enum class PoleForm { NONE, RAKIC, JM };
struct NamedMaterial {
    std::vector<std::string> names;
    double epsInf;
    PoleForm form;
    std::vector<double> params;
};

const std::vector<NamedMaterial>& named_materials() {
    static const std::vector<NamedMaterial> table = {
        {{"Au", "au", "AU"}, 1.0 + 1.0e-14, PoleForm::RAKIC,
         {9.03, 0.760, 0.053, 0.0, 0.024, 0.241, 0.415, 0.010, 0.345, 0.830, 0.071, 0.870, 2.969, 0.601, 2.494, 4.304, 4.384, 2.214, 13.32}},
        {{"Ag", "ag", "AG"}, 1.0 + 1.1e-14, PoleForm::RAKIC,
         {9.01, 0.845, 0.048, 0.0, 0.065, 3.886, 0.816, 0.124, 0.452, 4.481, 0.011, 0.065, 8.185, 0.840, 0.916, 9.083, 5.646, 2.419, 20.29}},
        {{"Al", "al", "AL"}, 1.0 + 1.2e-14, PoleForm::RAKIC,
         {14.98, 0.523, 0.047, 0.0, 0.227, 0.333, 0.162, 0.050, 0.312, 1.544, 0.166, 1.351, 1.808, 0.030, 3.382, 3.473}},
        {{"Cu", "cu", "CU"}, 1.0 + 1.3e-14, PoleForm::RAKIC,
         {10.83, 0.575, 0.030, 0.0, 0.061, 0.378, 0.291, 0.104, 1.056, 2.957, 0.723, 2.213, 5.300, 0.638, 4.305, 11.18}},
        {{"Be", "be", "BE"}, 1.0 + 1.4e-14, PoleForm::RAKIC,
         {18.51, 0.084, 0.035, 0.0, 0.031, 1.664, 0.100, 0.140, 3.395, 1.032, 0.530, 4.454, 3.183, 0.130, 1.802, 4.604}},
        {{"Cr", "cr", "CR"}, 1.0 + 1.5e-14, PoleForm::RAKIC,
         {10.75, 0.168, 0.047, 0.0, 0.151, 3.175, 0.121, 0.150, 1.305, 0.543, 1.149, 2.676, 1.970, 0.825, 1.335, 8.775}},
        {{"Ni", "ni", "NI"}, 1.0 + 1.6e-14, PoleForm::RAKIC,
         {15.92, 0.096, 0.048, 0.0, 0.100, 4.511, 0.174, 0.135, 1.334, 0.582, 0.106, 2.178, 1.597, 0.729, 6.292, 6.089}},
        {{"Pt", "pt", "PT"}, 1.0 + 1.7e-14, PoleForm::RAKIC,
         {9.59, 0.333, 0.080, 0.0, 0.191, 0.517, 0.780, 0.659, 1.838, 1.314, 0.547, 3.668, 3.141, 3.576, 8.517, 9.249}},
        {{"Pd", "pd", "PD"}, 1.0 + 1.8e-14, PoleForm::RAKIC,
         {9.72, 0.330, 0.008, 0.0, 0.649, 2.950, 0.336, 0.121, 0.555, 0.501, 0.638, 4.621, 1.659, 0.453, 3.236, 5.715}},
        {{"Ti", "ti", "TI"}, 1.0 + 1.9e-14, PoleForm::RAKIC,
         {7.29, 0.148, 0.082, 0.0, 0.899, 2.276, 0.777, 0.393, 2.518, 1.545, 0.187, 1.663, 2.509, 0.001, 1.762, 19.43}},
        {{"W", "w"}, 1.0 + 2.0e-14, PoleForm::RAKIC,
         {13.22, 0.206, 0.064, 0.0, 0.054, 0.530, 1.004, 0.166, 1.281, 1.917, 0.706, 3.332, 3.580, 2.590, 5.836, 7.498}},
        {{"TiO2"}, 6.20001, PoleForm::NONE, {}},
        {{"SiO2"}, 2.1025, PoleForm::NONE, {}},
        {{"Si"}, 11.8336, PoleForm::NONE, {}},
        {{"CdSe"}, 6.20, PoleForm::NONE, {}},
        {{"CdSeQD"}, 6.20, PoleForm::RAKIC, {2.03253, 0.65, 0.140, 2.03253}},
        {{"PbS"}, 17.20, PoleForm::NONE, {}},
        {{"PbSQD"}, 17.20, PoleForm::RAKIC, {1.45864, 5.00, 0.26, 1.45864}},
        {{"vac", "Vac", "VAC"}, 1.0, PoleForm::NONE, {}},
        {{"JM_Ag", "JM_ag", "JM_AG"}, 1.256, PoleForm::JM, {9.219, 1.0, 0.000, 0.0, 2.244, 0.133, 5.456, 0.187, 0.407, 2.014}},
        {{"JM_Au", "JM_au", "JM_AU"}, 5.513, PoleForm::JM, {9.013, 1.0, 0.000, 0.0, 1.857, 0.714, 3.658, 1.004, 0.399, 2.833}},
        {{"JM_Al", "JM_al", "JM_AL"}, 1.000 + 2.1e-14, PoleForm::JM, {14.344, 1.0, 0.651, 0.0, 4.283, 0.203, 1.645, 0.069, 0.036, 3.933}},
        {{"JM_Ga", "JM_ga", "JM_GA"}, 1.000 + 2.2e-14, PoleForm::JM, {9.954, 1.0, 1.796, 0.0, 30.615, 0.912, 1.863, 3.440, 0.215, 2.136}},
        {{"JM_Sn", "JM_sn", "JM_SN"}, 1.203, PoleForm::JM, {12.439, 1.0, 0.757, 0.0, 0.560, 1.546, 6.699, 0.902, 0.563, 4.011}},
        {{"JM_Tl", "JM_tl", "JM_TL"}, 1.456, PoleForm::JM, {6.314, 1.0, 0.000, 0.0, 0.527, 0.989, 5.332, 52.200, 0.763, 1.378}},
        {{"JM_Pb", "JM_pb", "JM_PB"}, 1.000 + 2.3e-14, PoleForm::JM, {9.210, 1.0, 0.157, 0.0, 1.602, 14.011, 16.755, 17.903, 1.138, 2.449}},
        {{"JM_Bi", "JM_bi", "JM_BI"}, 3.702, PoleForm::JM, {9.004, 1.0, 0.878, 0.0, 5.244, 1.833, 2.914, 5.161, 0.308, 1.484}},
    };
    return table;
}

// Oscillators of a named material's parameter set (getMetal / getMetalJM,
// parallelInputs.cpp:1186-1261): energies in eV to FDTD frequencies (ev2FDTD); a zero
// centre is the Drude term, given a 1e-20 eV centre. Rakic: sigma = f (wp / omega)^2,
// gamma_in = Gamma; JM: the Drude term as Rakic's with f = 1, the others sigma = f and
// gamma_in = 2 Gamma. The stored values are gamma_in pi and omega 2 pi, as for custom poles.
std::vector<Oscillator> named_poles(const NamedMaterial& m, double a) {
    std::vector<Oscillator> out;
    if (m.form == PoleForm::NONE) return out;
    auto ev2fdtd = [a](double ev) { return ev / 4.135666e-15 * a / kSpeedOfLight; };
    const std::vector<double>& par = m.params;
    const double wp = ev2fdtd(par[0]);
    for (std::size_t ii = 0; ii < (par.size() - 1) / 3; ++ii) {
        Oscillator osc;
        osc.dipOrE = DipOr::ISOTROPIC;
        osc.uVecDipE = {1.0, 1.0, 1.0};
        const double f = par[3 * ii + 1];
        const double GAM = ev2fdtd(par[3 * ii + 2]);
        double OMG = ev2fdtd(par[3 * ii + 3]);
        bool drude = false;
        if (OMG == 0.0) {
            drude = true;
            OMG = ev2fdtd(1.0e-20);
        }
        if (m.form == PoleForm::RAKIC) {
            osc.sigP = f * std::pow(wp / OMG, 2);
            osc.gam = GAM * M_PI;
        } else {
            osc.sigP = drude ? std::pow(wp / OMG, 2.0) : f;
            osc.gam = drude ? GAM * M_PI : 2.0 * GAM * M_PI;
        }
        osc.omg = OMG * 2.0 * M_PI;
        out.push_back(osc);
    }
    return out;
}

// parallelProgramInputs::ptreeToObject, parallelInputs.cpp:1263-1623 (custom materials,
// every shape of OBJECTS/Obj.hpp).
Object read_object(const JNode& node, const Inputs& ip) {
    Object o;
    o.loc = as_arr3(node, "loc");
    std::string material = node.get<std::string>("material");
    if (material != "custom") {
        const NamedMaterial* m = nullptr;
        for (const NamedMaterial& nm : named_materials())
            for (const std::string& n : nm.names)
                if (n == material) m = &nm;
        if (!m)
            throw InputError("The material name " + material +
                             " is not a predefined material. Please give me all the parameters or select from one of our predefined materials");
        o.epsInf = m->epsInf;
        o.pols = named_poles(*m, ip.a);
    } else {
        o.epsInf = node.get<double>("eps", 1.00);
        // a constant mu (parallelInputs.cpp:1283) enters the H-side coefficients; magnetic
        // poles (sigma_m) stay rejected below
        o.muInf = node.get<double>("mu", 1.0);
        if (node.get<double>("tellegen", 0.0) != 0.0)
            throw UnsupportedError("Tellegen media are not supported");
        for (auto& kv : node.child("pols").kids) {
            const JNode& pn = kv.second;
            // a tangential-isotropic pole needs relative electric and magnetic orientations
            // (parallelInputs.cpp:1290-1295); magnetic orientations are rejected below, so
            // with tanIso set the reference's own check is the one that applies
            if (pn.get<bool>("tanIso", false))
                throw InputError("Object can't be isotropic in tangential directions and unidirectional or isotropic");
            if (pn.get<bool>("molecular_trans", false)) throw UnsupportedError("molecular-transition poles are not supported");
            Oscillator osc;
            const std::string dipOrName = pn.get<std::string>("dipOrE", "isotropic");
            osc.dipOrE = string2dipor(dipOrName);
            if (string2dipor(pn.get<std::string>("dipOrM", "isotropic")) != DipOr::ISOTROPIC)
                throw UnsupportedError("magnetic dipole orientations are not supported");
            // dipoles relative to the surface normal (parallelInputs.cpp:1330-1357): polar
            // angle from the normal and azimuth in the tangent plane, fixed by the named forms
            double polAng = pn.get<double>("polAngRelNormE", 45.0);
            double azAng = pn.get<double>("azAngRelNormE", 45.0);
            if (dipOrName == "normal") {
                polAng = 0.0;
            } else if (dipOrName == "tangent") {
                polAng = 90.0;
            } else if (osc.dipOrE == DipOr::LONG_TAN) {
                polAng = 90.0;
                azAng = 0.0;
            } else if (osc.dipOrE == DipOr::LAT_TAN) {
                polAng = 90.0;
                azAng = 90.0;
            }
            osc.normW = std::cos(polAng * M_PI / 180.0);
            osc.latW = std::sin(polAng * M_PI / 180.0) * std::sin(azAng * M_PI / 180.0);
            osc.longW = std::sin(polAng * M_PI / 180.0) * std::cos(azAng * M_PI / 180.0);
            osc.gam = pn.get<double>("gamma") * M_PI;
            osc.omg = pn.get<double>("omega") * 2 * M_PI;
            osc.sigP = pn.get<double>("sigma_p", 0.0);
            if (pn.get<double>("sigma_m", 0.0) != 0.0) throw UnsupportedError("magnetic poles (sigma_m) are not supported");
            if (pn.get<double>("tau", 0.0) != 0.0) throw UnsupportedError("chiral poles (tau) are not supported");
            if (osc.dipOrE == DipOr::UNIDIRECTIONAL) {
                if (osc.sigP > 0.0) {
                    osc.uVecDipE = as_arr3(pn, "dirDipE");
                    double nrm = std::sqrt(std::accumulate(osc.uVecDipE.begin(), osc.uVecDipE.end(), 0.0,
                                                           [](double s, double v) { return s + v * v; }));
                    for (auto& v : osc.uVecDipE) v = v / nrm;
                } else {
                    osc.uVecDipE = {0.0, 0.0, 0.0};
                }
            } else {
                osc.uVecDipE = {1.0, 1.0, 1.0};
            }
            o.pols.push_back(osc);
        }
    }
    // unit vectors (parallelInputs.cpp:1439-1466)
    std::array<std::array<double, 3>, 3> uv{};
    const JNode& uvecs = node.child("unit_vectors");
    int cc = 0;
    for (auto& kv : uvecs.kids) {
        if (cc > 2) throw InputError("unit_vectors has more than three entries");
        uv[cc] = as_arr3(kv.second, "uvec");
        ++cc;
    }
    if (uvecs.size() == 0) {
        double orTheta = M_PI / 2.0 - node.get<double>("orTheta", 90.0) * M_PI / 180.0;
        double orPhi = -1.0 * node.get<double>("orPhi", 0.0) * M_PI / 180.0;
        if (ip.size[2] == 0) {
            uv[0] = {std::cos(orPhi), -1.0 * std::sin(orPhi), 0};
            uv[1] = {std::sin(orPhi), std::cos(orPhi), 0};
            uv[2] = {0.0, 0.0, 0};
        } else {
            uv[0] = {std::cos(orTheta) * std::cos(orPhi), -1.0 * std::cos(orTheta) * std::sin(orPhi), std::sin(orTheta)};
            uv[1] = {std::sin(orPhi), std::cos(orPhi), 0};
            uv[2] = {-1.0 * std::sin(orTheta) * std::cos(orPhi), std::sin(orTheta) * std::sin(orPhi), std::cos(orTheta)};
        }
    }
    // coordTransform_ rows (Obj.cpp:61-69): unit vector component / vector norm
    for (int ii = 0; ii < 3; ++ii) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += uv[ii][k] * uv[ii][k];
        for (int jj = 0; jj < 3; ++jj) {
            double dot = 0.0;
            for (int k = 0; k < 3; ++k) dot += uv[ii][k] * (k == jj ? 1.0 : 0.0);
            o.coord[ii * 3 + jj] = dot / std::sqrt(s);
        }
    }
    o.ML = node.child("Basis_Set").size() > 0;
    // shapes and their parameters (parallelInputs.cpp:1468-1622, string2shape :921-951)
    std::string s = node.get<std::string>("shape");
    auto geoTail = [&]() { o.geoML = o.geo; };
    if (s == "block") {
        o.geo = as_vector(node, "size");
        o.geo.push_back(node.get<double>("rad_curve", 0.0));
        if (o.geo.back() == 0.0) {
            o.shape = Shape::BLOCK;
        } else {
            // rounded_block (Obj.cpp:133-145): the centres of curvature of the eight corners
            o.shape = Shape::ROUNDED_BLOCK;
            const double rc = o.geo.back();
            for (int c = 0; c < 8; ++c)
                for (int k = 0; k < 3; ++k)
                    o.curveCens[c][k] = ((c >> k) & 1) ? -1.0 * o.geo[k] / 2.0 + rc : o.geo[k] / 2.0 - rc;
        }
        geoTail();
    } else if (s == "ellipsoid") {
        o.shape = Shape::ELLIPSOID;
        o.geo = as_vector(node, "size");
        o.cutNeg = as_arr3(node, "cut_neg", -1.0);
        o.cutPos = as_arr3(node, "cut_pos", 1.0);
        o.cutGlobal = as_arr3(node, "cut_global", 1.0);
        for (int nn = 0; nn < 3; ++nn)
            if (std::abs(o.cutNeg[nn]) > 1.0 || std::abs(o.cutPos[nn]) > 1.0 || std::abs(o.cutGlobal[nn]) > 1.0)
                throw InputError("abs(ellipsoid cutoff) must be <= 1.0");
        geoTail();
    } else if (s == "hemiellipsoid") {
        o.shape = Shape::HEMIELLIPSOID;
        o.geo = as_vector(node, "size");
        geoTail();
    } else if (s == "sphere" || s == "hemisphere") {
        o.shape = s == "sphere" ? Shape::SPHERE : Shape::HEMISPHERE;
        o.geo = {node.get<double>("radius", 0.0)};
        geoTail();
    } else if (s == "cylinder") {
        o.shape = Shape::CYLINDER;
        o.geo = {node.get<double>("radius", 0.0), node.get<double>("length", 0.0)};
        geoTail();
    } else if (s == "cone") {
        o.shape = Shape::CONE;
        const double rad1 = node.get<double>("radSmall", 0.0);
        const double rad2 = node.get<double>("radLarge", 0.0);
        if (rad2 <= rad1) throw InputError("radLarge for a cone must be greater than radSmall.");
        const double len = node.get<double>("height", 0.0);
        const double raiseAng = std::atan((rad2 - rad1) / len);
        o.geo = {rad2, len, rad2 * std::tan(raiseAng)};
        geoTail();
    } else if (s == "trapezoid_prism") {
        o.shape = Shape::TRI_PRISM;
        const double base1 = node.get<double>("base1", 0.0);
        const double base2 = node.get<double>("base2", 0.0);
        const double base = std::max(base1, base2);
        const double height = node.get<double>("height", 0.0);
        const double heightTri = base * 2.0 * height / (base1 - base2);
        std::array<std::array<double, 2>, 3> v = {{{0, 0.5 * heightTri}, {0.5 * base, -0.5 * heightTri}, {-0.5 * base, -0.5 * heightTri}}};
        o.geo = {std::abs(height / heightTri), 1.0, 1.0, node.get<double>("length", 0.0)};
        geoTail();
        setup_prism(o, v);
    } else if (s == "triangle_prism") {
        o.shape = Shape::TRI_PRISM;
        // the vertex form; any failure in it falls back to the base/height form, as the
        // reference's try block does
        bool done = false;
        const std::array<double, 3> loc0 = o.loc;
        try {
            const JNode& vl = node.child("vertLocs");
            std::vector<double> g = as_vector(node, "barry_center_cutoff", 1.0, 3);
            g.push_back(node.get<double>("length", 0.0));
            std::array<std::array<double, 2>, 3> v{};
            int cc = 0;
            for (auto& kv : vl.kids) {
                if (cc > 2) throw InputError("A triangle has exactly 3 verticies.");
                const std::array<double, 3> p3 = as_arr3(kv.second, "vert", 0.0);
                v[cc] = {p3[0], p3[1]};
                ++cc;
            }
            if (cc != 3) throw InputError("A triangle has exactly 3 verticies.");
            o.geo = g;
            geoTail();
            setup_prism(o, v);
            done = true;
        } catch (const std::exception&) {
            o.loc = loc0;
        }
        if (!done) {
            // base/height form (Obj.cpp:147-174): vertices (b/2, -h/2), (-b/2, -h/2), (0, h/2)
            const double base = node.get<double>("base", 0.0), height = node.get<double>("height", 0.0);
            o.geo = {base, height, 1.0, node.get<double>("length", 0.0)};
            geoTail();
            std::array<std::array<double, 2>, 3> v = {{{0.5 * base, -0.5 * height}, {-0.5 * base, -0.5 * height}, {0.0, 0.5 * height}}};
            setup_prism(o, v);
            o.geo = {1.0, 1.0, 1.0, o.geo[3]};
        }
    } else if (s == "ters_tip") {
        o.shape = Shape::TERS_TIP;
        o.geo = {2.0 * node.get<double>("rad_curve", 0.0), node.get<double>("base", 0.0), node.get<double>("length", 0.0)};
        o.radCen = {0.0, 0.0, -1.0 * o.geo[2] / 2.0 + o.geo[0] / 2.0};
        geoTail();
    } else if (s == "paraboloid") {
        o.shape = Shape::PARABOLOID;
        const double rc = node.get<double>("rad_curve", 0.0);
        o.geo = {node.get<double>("a", 1.0 / (2.0 * rc)), node.get<double>("b", 1.0 / (2.0 * rc)), node.get<double>("length", 0.0)};
        geoTail();
    } else if (s == "torus") {
        o.shape = Shape::TORUS;
        o.geo = {node.get<double>("rad_Ring", 0.0), node.get<double>("rad_CrossSec", 0.0),
                 node.get<double>("phiMin", 0.0) * M_PI / 180.0, node.get<double>("phiMax", 360.0) * M_PI / 180.0};
        geoTail();
    } else if (s == "tetrahedron") {
        o.shape = Shape::TETRAHEDRON;
        if (o.ML) throw UnsupportedError("emitters in a tetrahedron are not supported");
        bool done = false;
        const std::array<double, 3> loc0 = o.loc;
        const std::array<double, 9> coord0 = o.coord;
        try {
            const JNode& vl = node.child("vertLocs");
            std::vector<double> g = as_vector(node, "barry_center_cutoff", 1.0, 4);
            int cc = 0;
            for (auto& kv : vl.kids) {
                if (cc > 3) throw InputError("A tetrahedron has exactly 4 verticies.");
                o.verts[cc] = as_arr3(kv.second, "vert");
                ++cc;
            }
            if (cc != 4) throw InputError("A tetrahedron has exactly 4 verticies.");
            // real-space vertices: location and unit vectors are reset (parallelInputs.cpp:1602-1606)
            o.loc = {0.0, 0.0, 0.0};
            o.coord = {1, 0, 0, 0, 1, 0, 0, 0, 1};
            o.geo = g;
            geoTail();
            setup_tetrahedron(o);
            done = true;
        } catch (const std::exception&) {
            o.loc = loc0;
            o.coord = coord0;
        }
        if (!done) {
            // regular tetrahedron of side sideLen about the location (Obj.cpp:215-252)
            o.geo = {node.get<double>("sideLen", 2.0 / std::sqrt(3.0) * node.get<double>("perpBiSect", -1.0))};
            if (o.geo[0] == -1) throw InputError("please give a side length or prepindicular bisector length for the tetrahedron.");
            o.geo.push_back(node.get<double>("height", std::sqrt(2.0 / 3.0) * o.geo[0]));
            geoTail();
            const double unit[4][3] = {{std::sqrt(8.0 / 9.0), 0, -1.0 / 3.0},
                                       {-1.0 * std::sqrt(2.0 / 9.0), std::sqrt(2.0 / 3.0), -1.0 / 3.0},
                                       {-1.0 * std::sqrt(2.0 / 9.0), -1.0 * std::sqrt(2.0 / 3.0), -1.0 / 3.0},
                                       {0, 0, 1}};
            for (int v = 0; v < 4; ++v) {
                for (int i = 0; i < 3; ++i) {
                    double t = 0.0;
                    for (int k = 0; k < 3; ++k) t += o.coord[i * 3 + k] * unit[v][k];
                    o.verts[v][i] = t;
                }
                for (int i = 0; i < 3; ++i) o.verts[v][i] *= o.geo[0] * std::sqrt(3.0 / 8.0);
                for (int i = 0; i < 3; ++i) o.verts[v][i] = 1.0 * o.loc[i] + o.verts[v][i];
            }
            setup_tetrahedron(o);
            // the fourth cut-off: the barycentric weight of vertex 4 at the requested height
            const double heightRat = (o.geo[1] / (o.geo[0] * std::sqrt(2.0 / 3.0)) * (5.0 / 4.0)) - 1.0 / 4.0;
            double v4[3];
            for (int i = 0; i < 3; ++i) v4[i] = heightRat * o.verts[3][i] + o.loc[i];
            const std::array<double, 4> b = to_bary<4>(o.invVert, v4);
            o.geo = {1.0, 1.0, 1.0, b[3]};
        }
    } else {
        throw InputError("A shape in the ObjectList is not defined in the code");
    }
    return o;
}

// Adds buffer cells around an emitter object so that the polarisation points, which sit
// between grid points, are inside it (Obj::addMLBuff, OBJECTS/Obj.hpp:537,653,776,949).
void add_ml_buffer(Object& o, double d) {
    auto add = [&](std::initializer_list<int> idx) {
        for (int i : idx) o.geoML[static_cast<std::size_t>(i)] += 3.0 * d;
    };
    switch (o.shape) {
        case Shape::SPHERE:
        case Shape::HEMISPHERE: add({0}); break;
        case Shape::BLOCK:
        case Shape::ROUNDED_BLOCK:
        case Shape::ELLIPSOID:
        case Shape::HEMIELLIPSOID:
        case Shape::TRI_PRISM:
        case Shape::TERS_TIP: add({0, 1, 2}); break;
        case Shape::CONE: add({1}); break;
        case Shape::CYLINDER:
        case Shape::PARABOLOID:
        case Shape::TORUS: add({0, 1}); break;
        case Shape::TETRAHEDRON: break;  // emitters in a tetrahedron are rejected when read
    }
}

// Inhomogeneous-broadening weight functions (UTIL/ML_Dist_Fxn.hpp:14-50): the normal density,
// its log-normal, skew-normal, exponential-power and generalised skew-normal forms.
static double norm_dist(double x, double cen, double w) {
    return 1.0 / std::sqrt(2 * M_PI * std::pow(w, 2.0)) * std::exp(-1.0 * std::pow(x - cen, 2.0) / (2.0 * std::pow(w, 2.0)));
}
static double log_norm_dist(double x, double cen, double w) {
    return (x <= cen) ? 0.0
                      : 1.0 / std::sqrt(2 * M_PI * std::pow(w * x, 2.0)) *
                            std::exp(-1.0 * std::pow(std::log(x) - cen, 2.0) / (2.0 * std::pow(w, 2.0)));
}
static double skew_norm_dist(double x, double cen, double w, double skew) {
    return norm_dist(x, cen, w) * 0.5 * (1.0 + std::erf(skew * (x - cen) / (std::sqrt(2.0) * w)));
}
// exponential-power (generalised normal) density of shape s: s / (2 w Gamma(1/s)) exp(-(|x - c| / w)^s)
static double exp_pow_dist(double x, double cen, double w, double s) {
    return s / (2 * w * std::tgamma(1.0 / s)) * std::exp(-1.0 * std::pow(std::abs(x - cen) / w, s));
}
// generalised skew-normal of shape k as the reference writes it: zero beyond c + w / k, else
// the standard normal density at y = -log(1 - k^2 (x - c) / w) / k over (w - k (x - c))
// (the reference's argument carries k twice); the normal density for k = 0
static double gen_skew_norm_dist(double x, double cen, double w, double k) {
    if (k == 0.0) return norm_dist(x, cen, w);
    if ((k < 0 && x < cen + w / k) || (k > 0 && x > cen + w / k)) return 0.0;
    const double y = -1.0 / k * std::log(1 - k * (k * (x - cen) / w));
    return norm_dist(y, 0.0, 1.0) / (w - k * (x - cen));
}

enum class LevelDist { GAUSSIAN, DELTA, SKEW_NORMAL, LOG_NORMAL, EXP_POW, GEN_SKEW_NORMAL };

// parallelProgramInputs::string2dist, parallelInputs.cpp:903-919
static LevelDist string2dist(const std::string& d) {
    if (d == "Gaussian" || d == "gaussian") return LevelDist::GAUSSIAN;
    if (d == "delta_fxn" || d == "Delta_fxn" || d == "Delta_Fxn" || d == "delta_Fxn" || d == "DeltaFxn") return LevelDist::DELTA;
    if (d == "skew_normal" || d == "Skew_Normal" || d == "Skew_normal" || d == "skew_Normal") return LevelDist::SKEW_NORMAL;
    if (d == "log_normal" || d == "Log_Normal" || d == "Log_normal" || d == "log_Normal") return LevelDist::LOG_NORMAL;
    if (d == "exp_pow" || d == "Exp_Pow" || d == "Exp_pow" || d == "exp_Pow") return LevelDist::EXP_POW;
    if (d == "gen_skew_normal" || d == "Gen_Skew_Normal" || d == "Gen_Skew_normal" || d == "gen_skew_Normal")
        return LevelDist::GEN_SKEW_NORMAL;
    throw InputError("The distribution type " + d + " is not defined, please define it for me.");
}

// The emitter part of an object (parallelInputs.cpp:425-662): removes the points of earlier
// emitters that this object covers, then, when the object has a basis set, reads its levels,
// couplings, relaxation and outputs, lists its grid points and buffers its geometry.
void read_emitter(const JNode& node, Object& o, Inputs& ip) {
    std::vector<std::array<int, 2>> basis;
    for (auto& kv : node.child("Basis_Set").kids)
        basis.push_back({kv.second.get<int>("l"), kv.second.get<int>("m")});
    const int nx = find_pt(ip.size[0], ip.d[0]) + 1;
    const int ny = find_pt(ip.size[1], ip.d[1]) + 1;
    const int nz = find_pt(ip.size[2], ip.d[2]) + 1;
    const double dminAll = *std::min_element(ip.d.begin(), ip.d.end());
    // points of earlier emitters inside this object are dropped (the position used here is
    // one cell below the one used when the points were listed, as in the reference)
    for (auto& em : ip.emitters) {
        for (std::size_t ll = 0; ll < em.locs.size(); ++ll) {
            std::array<double, 3> loc = {(em.locs[ll][0] - (nx - 1) / 2.0 - 1) * ip.d[0],
                                         (em.locs[ll][1] - (ny - 1) / 2.0 - 1) * ip.d[1],
                                         (em.locs[ll][2] - (nz - 1) / 2.0 - 1) * ip.d[2]};
            if (o.isObj(loc, dminAll, o.geo)) {
                em.locs.erase(em.locs.begin() + ll);
                --ll;
            }
        }
    }
    if (basis.empty()) return;
    // A second emitter object: the reference pools the energy levels of every emitter
    // object (qeELevs_, parallelInputs.cpp:578) and builds each object's Hamiltonians from
    // the pooled list (parallelFDTDField.cpp:423), whose diagonal then disagrees with the
    // ensemble energies, and parallelQE's constructor throws (ML/parallelQE.hpp:220-228).
    if (!ip.emitters.empty())
        throw InputError("The energy for the weight and the Hamiltonian at index 0 do not match, please fix this error. "
                         "(a second emitter object: the reference pools the energy levels of all emitter objects)");
    const double eConv = kElementaryCharge * kEps0 * std::pow(kSpeedOfLight / ip.I0, 2) / ip.a;
    EmitterSpec em;
    em.object = static_cast<int>(ip.objects.size());
    em.basis = basis;
    em.molDen = node.get<double>("mol_den", 1.0);
    const int numElProportion = node.get<int>("numElectorn", 1);
    for (auto& kv : node.child("Energy_Levels").kids) {
        const JNode& lev = kv.second;
        EnergyLevel level;
        std::vector<double> eCen = as_vector(lev, "E_cen");
        for (auto& e : eCen) e *= eConv;
        std::vector<double> wVec = as_vector(lev, "weights", 1.0, static_cast<int>(eCen.size()));
        const LevelDist dist = string2dist(lev.get<std::string>("distribution", "Delta_Fxn"));
        const int nstates = lev.get<int>("nstates", 1);
        const double top = lev.get<double>("highEdge", eCen[0] / eConv + lev.get<double>("BandWith", 0.0) / 2.0) * eConv;
        const double bot = lev.get<double>("lowEdge", eCen[0] / eConv - lev.get<double>("BandWith", 0.0) / 2.0) * eConv;
        const int numLevs = lev.get<int>("levs_described", 1);
        if (dist == LevelDist::DELTA || nstates == 1) {
            if (nstates > 1) throw InputError("The number of states is greater than one for a delta function distribution.");
            level.weights = wVec;
            level.energyStates = eCen;
        } else {
            double weightSum = 0.0;
            for (int n = 0; n < nstates; ++n) level.energyStates.push_back(bot + n * (top - bot) / (nstates - 1.0));
            for (double es : level.energyStates) {
                std::vector<double> width = as_vector(lev, "dist_width");
                for (auto& w : width) w *= eConv;
                if (width.size() != eCen.size())
                    throw InputError("The center frequency and distribution width is not the same size.");
                double weight = 0.0;
                if (dist == LevelDist::GAUSSIAN) {
                    for (std::size_t i = 0; i < width.size(); ++i) weight += wVec[i] * norm_dist(es, eCen[i], width[i]);
                } else if (dist == LevelDist::LOG_NORMAL) {
                    for (std::size_t i = 0; i < width.size(); ++i) weight += wVec[i] * log_norm_dist(es, eCen[i], width[i]);
                } else if (dist == LevelDist::SKEW_NORMAL) {
                    std::vector<double> skew = as_vector(lev, "skew_factor");
                    if (skew.size() != eCen.size())
                        throw InputError("The center frequency and skew factor do not have the same size.");
                    for (std::size_t i = 0; i < width.size(); ++i)
                        weight += wVec[i] * skew_norm_dist(es, eCen[i], width[i], skew[i]);
                } else {
                    // GEN_SKEW_NORMAL and EXP_POW: one shape factor per centre
                    std::vector<double> shape = as_vector(lev, "shape_factor");
                    if (shape.size() != eCen.size())
                        throw InputError("The center frequency and shape factor do not have the same size.");
                    for (std::size_t i = 0; i < width.size(); ++i)
                        weight += wVec[i] * (dist == LevelDist::EXP_POW ? exp_pow_dist(es, eCen[i], width[i], shape[i])
                                                                        : gen_skew_norm_dist(es, eCen[i], width[i], shape[i]));
                }
                level.weights.push_back(weight);
                weightSum += weight;
            }
            for (auto& w : level.weights) w /= weightSum / static_cast<double>(numElProportion);
        }
        level.levDescribed = numLevs;
        ip.qeELevs.push_back(level);
    }
    for (auto& kv : node.child("couplings").kids)
        em.couplings.push_back(kv.second.value<double>() * 1.0e-21 / std::pow(ip.a, 2.0) / ip.I0);
    for (auto& kv : node.child("gam").kids) {
        std::vector<double> g;
        for (auto& gg : kv.second.child("g").kids) g.push_back(gg.second.value<double>() * ip.a / kSpeedOfLight);
        em.gam.push_back(g);
    }
    // grid points of the object (parallelInputs.cpp:596-614), in (z, y, x) order; the z
    // planes are scanned in parallel and concatenated in order
    {
        std::vector<std::vector<std::array<int, 3>>> plane(static_cast<std::size_t>(std::max(nz, 0)));
#pragma omp parallel for schedule(dynamic, 1)
        for (int zz = 0; zz < nz; ++zz)
            for (int yy = 0; yy < ny; ++yy)
                for (int xx = 0; xx < nx; ++xx) {
                    std::array<double, 3> pt = {(xx - (nx - 1) / 2.0) * ip.d[0], (yy - (ny - 1) / 2.0) * ip.d[1],
                                                (zz - (nz - 1) / 2.0) * ip.d[2]};
                    if (o.isObj(pt, dminAll, o.geo)) plane[zz].push_back({xx, yy, zz});
                }
        for (auto& pl : plane) em.locs.insert(em.locs.end(), pl.begin(), pl.end());
        if (o.baryFault->load()) throw InputError("The sum of the boundary checks for a triangular base does not equal the determinant of the verticies");
    }
    for (auto& kv : node.child("RelaxationOperators").kids) {
        RelaxOp r;
        r.n0 = kv.second.get<int>("state_i");
        r.nf = kv.second.get<int>("state_f");
        r.rate = kv.second.get<double>("rate") * ip.a / kSpeedOfLight;
        r.dephasing = kv.second.get<double>("dephasing_rate", 0.0) * ip.a / kSpeedOfLight;
        em.relax.push_back(r);
    }
    // per-cell dipoles (extension; see EmitterSpec)
    {
        const std::string orient = node.get<std::string>("dipole_orientation", "");
        const std::vector<double> scale = node.has("dipole_scale_range") ? as_vector(node, "dipole_scale_range") : std::vector<double>{};
        if (!orient.empty() || !scale.empty()) {
            if (!orient.empty() && orient != "random" && orient != "z")
                throw InputError("dipole_orientation must be \"random\" or \"z\"");
            if (!scale.empty() && (scale.size() != 2 || !(scale[0] > 0.0) || scale[1] < scale[0]))
                throw InputError("dipole_scale_range must be two values 0 < a <= b");
            em.cellDipole = true;
            em.randomDirection = orient == "random";
            if (!scale.empty()) em.dipoleScale = {scale[0], scale[1]};
            em.dipoleSeed = static_cast<unsigned long long>(node.get<double>("dipole_seed", 0.0));
        }
    }
    em.outputPol = node.get<bool>("output_pol", false);
    if (em.outputPol) em.polFile = node.get<std::string>("output_pol_filename");
    for (auto& kv : node.child("dtc_levs").kids) em.dtcLevs.push_back(kv.second.value<int>());
    em.dtcTimeInt = node.get<int>("levDTC_timeInt", 1);
    const std::string base = node.get<std::string>("dtc_pop_fname_base", "output_data/qe_");
    for (int lv : em.dtcLevs)
        em.dtcFiles.push_back(base + std::to_string(ip.emitters.size()) + "_level_" + std::to_string(lv) + ".dat");
    add_ml_buffer(o, *std::max_element(ip.d.begin(), ip.d.end()));
    ip.emitters.push_back(em);
}

std::vector<double> read_freq_list(const JNode& n, const char* what) {
    double fCen = n.get<double>("fcen", -1.0);
    double fWidth = n.get<double>("fwidth", -1.0);
    double lamL = n.get<double>("lamL", -1.0);
    double lamR = n.get<double>("lamR", -1.0);
    int nFreq = n.get<int>("nfreq", -1);
    if (nFreq < 1) throw InputError(std::string(what) + " regions need a number of frequencies");
    std::vector<double> fl(nFreq, 0.0);
    if (fCen != -1.0 && fWidth != -1.0) {
        if (lamL != -1.0 && lamR != -1.0) throw InputError("Both a freq and wavelength range is defined");
        double dOmg = fWidth / static_cast<double>(nFreq - 1);
        for (int ii = 0; ii < nFreq; ++ii) fl[ii] = (fCen - fWidth / 2.0 + ii * dOmg) * 2.0 * M_PI;
    } else if (lamL != -1.0 && lamR != -1.0) {
        double dLam = (lamR - lamL) / static_cast<double>(nFreq - 1);
        for (int ii = 0; ii < nFreq; ++ii) fl[ii] = 2.0 * M_PI / (lamL + ii * dLam);
    } else {
        throw InputError(std::string(what) + " needs fcen and fwidth or lamL and lamR");
    }
    return fl;
}

// One TFSF surface (parallelInputs.cpp:219-408): the box in grid points (odd sizes
// unless the box is a plane), the propagation vector m from the angles or the angles
// from m, the pulses with the amplitude appended as (0, Emax)
// (parallelFDTDField.cpp:648), the polarisation and the 1-D CPML parameters.
void read_tfsf(const JNode& tn, Inputs& ip) {
    TfsfSpec t;
    const std::array<double, 3> tempSz = as_arr3(tn, "size");
    for (int i = 0; i < 3; ++i) t.sz[i] = find_pt(tempSz[i], ip.d[i]) + 1;
    const bool anyOne = t.sz[0] == 1 || t.sz[1] == 1 || t.sz[2] == 1;
    if ((ip.size[2] == 0 && t.sz[0] != 1 && t.sz[1] != 1) || (ip.size[2] != 0.0 && !anyOne))
        for (int& v : t.sz) v -= (v - 1) % 2;
    const std::array<double, 3> loc = as_arr3(tn, "loc");
    for (int i = 0; i < 3; ++i)
        t.loc[i] = (ip.size[i] != 0.0) ? find_pt(loc[i] + ip.size[i] / 2.0, ip.d[i]) - (t.sz[i] - (t.sz[i] % 2)) / 2 : 0;
    for (int i = 0; i < 3; ++i)
        if (ip.size[i] > 0.0 && (t.loc[i] + t.sz[i] / 2 > find_pt(ip.size[i], ip.d[i]) || t.loc[i] < 0))
            if (t.loc[i] + t.sz[i] / 2.0 != 1) throw InputError("A TFSF surface is outside the FDTD cell.");
    if (tn.has("m") && tn.child("m").size() > 0) {
        int i = 0;
        for (auto& mk : tn.child("m").kids) {
            if (i < 3) t.m[i] = mk.second.value<int>();
            ++i;
        }
        const int nz = (t.m[0] != 0) + (t.m[1] != 0) + (t.m[2] != 0);
        if (nz == 1)
            for (int& v : t.m)
                if (v != 0) v /= std::abs(v);
        t.phi = (t.m[0] == 0) ? ((t.m[1] > 0) ? M_PI / 2.0 : -1.0 * M_PI / 2.0)
                              : std::atan(t.m[1] * ip.d[0] / (t.m[0] * ip.d[1]));
        if (t.m[0] < 0) t.phi += M_PI;
        else if (t.m[1] < 0) t.phi += 2.0 * M_PI;
        t.theta = (t.m[2] == 0) ? M_PI / 2.0
                                : std::atan(std::sqrt(std::pow(t.m[1] / ip.d[1], 2.0) + std::pow(t.m[0] / ip.d[0], 2.0)) /
                                            (t.m[2] / ip.d[2]));
        if (t.m[2] < 0) t.theta += M_PI;
        t.psi = M_PI * tn.get<double>("psi", 90.0) / 180.0;
    } else {
        t.m = {0, 0, 0};
        t.theta = M_PI * tn.get<double>("theta", 90.0) / 180.0;
        if (t.theta < 0 || t.theta > M_PI) throw InputError("The theta value for the TFSF surfaces must be between 0 and 180 degrees.");
        t.phi = M_PI * tn.get<double>("phi", 90.0) / 180.0;
        t.psi = M_PI * tn.get<double>("psi", 90.0) / 180.0;
        if (ip.size[2] == 0.0) {
            t.theta = M_PI / 2.0;
            t.psi = (ip.pol == Pol::EZ || ip.pol == Pol::HX || ip.pol == Pol::HY) ? M_PI / 2.0 : 0.0;
        }
        if (std::fmod(t.theta, M_PI) == 0.0) t.m[2] = t.theta == 0 ? 1 : -1;
        else if (std::fmod(t.phi, M_PI) == 0.0) t.m[0] = (std::fmod(t.phi, 2 * M_PI) == 0.0) ? 1 : -1;
        else if (std::fmod(t.phi, M_PI / 2.0) == 0.0) t.m[1] = (std::fmod(t.phi, 2 * M_PI) == M_PI / 2.0) ? 1 : -1;
    }
    if (t.m[0] == 0 && t.m[1] == 0 && t.m[2] == 0) throw InputError("TFSF surface must have a direction of propgation.");
    for (auto& pk : tn.child("PulseList").kids) {
        PulseSpec p = read_pulse(pk.second, ip.a, ip.I0);
        p.param.back() = cplx(0.0, std::real(p.param.back()));
        t.pulses.push_back(p);
    }
    t.circPol = string2pol(tn.get<std::string>("circPol", "Ex"));
    t.kRatio = tn.get<double>("ellpiticalKRat", 1.0);
    t.pmlThick = tn.get<int>("pmlThick", 20);
    t.pmlAMax = tn.get<double>("pmlAMax", 0.0);
    t.pmlM = tn.get<double>("pmlM", ip.pmlM);
    t.pmlMa = tn.get<double>("pmlMa", ip.pmlMa);
    ip.tfsf.push_back(t);
}

}  // namespace

cplx PulseSpec::value(double tt) const {
    // UTIL/PulseFxn.hpp:19-89
    const std::vector<cplx>& p = param;
    switch (shape) {
        case PulseShape::GAUSSIAN:
            return (tt <= std::real(p[2])) ? p[4] * std::exp(p[0] * tt - (std::pow((tt - p[3]) / p[1], 2.0) / 2.0)) : cplx(0.0);
        case PulseShape::CONTINUOUS:
            return p[1] * std::exp(p[0] * tt);
        case PulseShape::RAMP_CONT:
            return (std::abs(p[2] * p[1] * tt) <= std::abs(p[2])) ? std::abs(p[1] * tt) * p[2] * std::exp(p[0] * tt)
                                                                    : p[2] * std::exp(p[0] * tt);
        case PulseShape::BH:
            return (std::real(p[2] - p[1] / 2.0) <= tt && tt <= std::real(p[2] + p[1] / 2.0))
                       ? p[7] * std::exp(p[0] * (tt - p[2])) *
                             (p[3] + p[4] * std::cos(2.0 * M_PI * (tt - p[2]) / p[1]) +
                              p[5] * std::cos(4.0 * M_PI * (tt - p[2]) / p[1]) +
                              p[6] * std::cos(6.0 * M_PI * (tt - p[2]) / p[1]))
                       : cplx(0.0);
        case PulseShape::RECT:
            return (tt < std::real(p[1] + p[0]) && tt > std::real(p[1] - p[0]))
                       ? p[4] / (std::pow(2.0 * (tt - p[1]) / p[0], p[2]) + 1.0) * (std::exp(p[3] * (tt - p[1])))
                       : cplx(0.0);
        case PulseShape::RICKER:
            return (tt < std::real(p[2] * p[1] / p[0]))
                       ? p[3] * (1.0 - 2.0 * std::pow(M_PI * (tt * p[0] - p[1]), 2.0)) *
                             std::exp(-std::pow(M_PI * (tt * p[0] - p[1]), 2.0))
                       : cplx(0.0);
    }
    return 0.0;
}

Inputs read_inputs(const JNode& IP, const std::string& filename) {
    Inputs ip;
    ip.filename = filename;
    // parallelInputs.cpp:14-27
    if (IP.get<bool>("CompCell.PBC", false)) throw UnsupportedError("periodic boundaries are not supported");
    if (IP.get<bool>("CompCell.cplxFields", false)) throw UnsupportedError("complex fields are not supported");
    ip.pol = string2pol(IP.get<std::string>("CompCell.pol"));
    ip.res = IP.get<int>("CompCell.res", -1);
    ip.courant = IP.get<double>("CompCell.courant", 0.5);
    ip.a = IP.get<double>("CompCell.a", 1e-7);
    ip.tMax = IP.get<double>("CompCell.tLim");
    ip.I0 = IP.get<double>("CompCell.I0", ip.a * kEps0 * kSpeedOfLight);
    ip.size = as_arr3(IP, "CompCell.size");
    ip.d = as_arr3(IP, "CompCell.stepSize", 1.0 / ip.res);
    ip.dt = IP.get<double>("CompCell.dt", ip.courant / std::sqrt(1.0 / (ip.d[0] * ip.d[0]) + 1.0 / (ip.d[1] * ip.d[1]) +
                                                                   1.0 / (ip.d[2] * ip.d[2])));
    ip.pmlSigOptRat = IP.get<double>("PML.sigOptRat", 1.0);
    ip.pmlKappaMax = IP.get<double>("PML.kappaMax", 1.0);
    ip.pmlAMax = IP.get<double>("PML.aMax", 0.00);
    ip.pmlMa = IP.get<double>("PML.ma", 1.0);
    ip.pmlM = IP.get<double>("PML.m", 3.0);
    // parallelInputs.cpp:96-107
    if (ip.d[0] < 0 || ip.d[1] < 0 || ip.d[2] < 0) throw InputError("Please define a positive step size.");
    double stab = 0.0;
    for (double dd : ip.d) stab += 1.0 / (dd * dd);
    if (ip.dt > 1.0 / std::sqrt(stab)) throw InputError("Time step is larger than the stable time step for the calculation.");
    std::array<double, 3> pmlT = as_arr3(IP, "PML.thickness");
    for (int ii = 0; ii < 3; ++ii) {
        if (pmlT[ii] * 2 > ip.size[ii]) throw InputError("PML size is larger than the cell size");
        ip.pmlThickness[ii] = find_pt(pmlT[ii], ip.d[ii]);
    }
    // Sources, parallelInputs.cpp:114-216
    for (auto& kv : IP.child("SourceList").kids) {
        const JNode& sn = kv.second;
        SourceSpec s;
        s.pol = string2pol(sn.get<std::string>("pol"));
        for (auto& pk : sn.child("PulseList").kids) s.pulses.push_back(read_pulse(pk.second, ip.a, ip.I0));
        std::array<double, 3> tempSz = as_arr3(sn, "size");
        for (int cc = 0; cc < 3; ++cc) s.sz[cc] = find_pt(tempSz[cc], ip.d[cc]) + 1;
        // "psi" and "ellpiticalKRat" of an L/R source only feed prefactors that its pulses
        // never read (setup.cpp, buildSources, says why); "theta" is not read.
        s.phi = sn.get<double>("phi", 90);
        std::array<double, 3> loc = as_arr3(sn, "loc");
        for (int i = 0; i < 3; ++i) {
            if (loc[i] + tempSz[i] / 2.0 > ip.size[i] / 2.0 || loc[i] - tempSz[i] / 2.0 < -1.0 * ip.size[i] / 2.0)
                throw InputError("The source is at least partially outside the FDTD Cell");
            if (s.phi == 90 || s.phi == 180 || s.phi == 270 || s.phi == 0)
                s.loc[i] = find_pt(loc[i] + ip.size[i] / 2.0 - tempSz[i] / 2.0, ip.d[i]);
            else
                s.loc[i] = find_pt(loc[i] + ip.size[i] / 2.0, ip.d[i]);
        }
        ip.sources.push_back(s);
    }
    // TFSF surfaces, parallelInputs.cpp:219-408
    for (auto& kv : IP.child("TFSF").kids) read_tfsf(kv.second, ip);
    // Objects, parallelInputs.cpp:410-666; objArr_[0] is the vacuum block of the whole cell
    ip.objects.push_back(make_vacuum_block(ip.size));
    for (auto& kv : IP.child("ObjectList").kids) {
        Object o = read_object(kv.second, ip);
        read_emitter(kv.second, o, ip);
        ip.objects.push_back(o);
    }
    // Detectors, parallelInputs.cpp:667-755
    int ii = 0;
    for (auto& kv : IP.child("DetectorList").kids) {
        const JNode& dn = kv.second;
        DetectorSpec d;
        d.outputMaps = dn.get<bool>("output_map", false);
        d.type = string2out(dn.get<std::string>("type"));
        d.name = dn.get<std::string>("fname") + "_field_" + std::to_string(ii) + ".dat";
        ++ii;
        std::string cls = dn.get<std::string>("dtc_class", "cout");
        if (cls == "txt") d.cls = DtcClass::TXT;
        else if (cls == "bin") d.cls = DtcClass::BIN;
        else if (cls == "freq") d.cls = DtcClass::FREQ;
        else if (cls == "cout" || cls == "bmp") throw UnsupportedError("detector class '" + cls + "' is not supported");
        else throw InputError("DTCCLASS (DetectorList.class) for input file is not defined");

        d.SI = dn.get<bool>("SI", true);
        d.timeInt = dn.get<double>("Time_Interval", ip.dt);
        std::array<double, 3> tempSz = as_arr3(dn, "size");
        for (int cc = 0; cc < 3; ++cc) d.sz[cc] = find_pt(tempSz[cc], ip.d[cc]) + 1;
        std::array<double, 3> loc = as_arr3(dn, "loc");
        for (int i = 0; i < 3; ++i) {
            if (loc[i] - tempSz[i] / 2.0 < -1.0 * ip.size[i] / 2.0 || loc[i] + tempSz[i] / 2.0 > ip.size[i] / 2.0)
                throw InputError("A detector is outside the FDTD cell.");
            d.loc[i] = find_pt(loc[i] + ip.size[i] / 2.0 - tempSz[i] / 2.0, ip.d[i]);
        }
        if (d.cls == DtcClass::FREQ) d.freqList = read_freq_list(dn, "The freq detector");
        ip.detectors.push_back(d);
    }
    // Flux regions, parallelInputs.cpp:756-838
    for (auto& kv : IP.child("FluxList").kids) {
        const JNode& fn = kv.second;
        FluxSpec f;
        f.name = fn.get<std::string>("name");
        std::array<double, 3> tempSz = as_arr3(fn, "size");
        for (int cc = 0; cc < 3; ++cc) f.sz[cc] = find_pt(tempSz[cc], ip.d[cc]) + 1;
        std::array<double, 3> loc = as_arr3(fn, "loc");
        for (int i = 0; i < 3; ++i) {
            if (loc[i] - tempSz[i] / 2.0 < -1.0 * ip.size[i] || loc[i] + tempSz[i] / 2.0 > ip.size[i])
                throw InputError("A flux region is outside the FDTD cell.");
            f.loc[i] = find_pt(loc[i] + ip.size[i] / 2.0 - tempSz[i] / 2, ip.d[i]);
        }
        f.weight = fn.get<double>("weight", 1.0);
        f.timeInt = static_cast<int>(std::floor(fn.get<double>("Time_Interval", ip.dt) / (ip.dt) + 0.50));
        if (f.timeInt <= 0) f.timeInt = 1;
        f.freqList = read_freq_list(fn, "flux");
        f.SI = fn.get<bool>("SI", false);
        f.crossSec = fn.get<bool>("cross_sec", false);
        f.incdFile = fn.get<std::string>("incd_fileds", "");
        f.save = fn.get<bool>("save", false);
        f.load = fn.get<bool>("load", false);
        if (f.load && f.incdFile == "")
            throw InputError("Trying to load in file without a valid path, in the " + std::to_string(ip.fluxes.size()) +
                             " flux detector");
        ip.fluxes.push_back(f);
    }
    return ip;
}

Inputs read_inputs_file(const std::string& path) { return read_inputs(parse_json_file(path), path); }

// Obj::setUpConsts (Obj.cpp:299-370), electric poles only
void Object::setUpConsts(double dt) {
    alpha.clear();
    xi.clear();
    gamma.clear();
    alphaInc.clear();
    dipOr.clear();
    dipE.clear();
    dipW.clear();
    orDip = false;
    for (auto& p : pols) {
        if (p.dipOrE != DipOr::ISOTROPIC) orDip = true;
        if (std::abs(p.sigP) != 0.0) {
            dipOr.push_back(p.dipOrE);
            dipE.push_back(p.uVecDipE);
            dipW.push_back({p.normW, p.latW, p.longW});
            alpha.push_back(((2 - std::pow(p.omg * dt, 2.0)) / (1 + p.gam * dt)));
            xi.push_back(((p.gam * dt - 1) / (1 + p.gam * dt)));
            gamma.push_back(((p.sigP * std::pow(p.omg * dt, 2.0)) / (1 + p.gam * dt)));
            alphaInc.push_back(-1.0 * std::pow(p.omg * dt, 2.0) / (1 + p.gam * dt));
        }
    }
}

// Shape tests, Obj.cpp:373-540 (isObj of every shape), with the reference's tolerances and
// arithmetic as written (including its quirks: the cone's radius test compares a distance
// with a squared length, the TERS tip takes the cosine of its apex diameter, and the
// torus's azimuth is NaN on its axis, where every test against it is false).
bool Object::isObj(const std::array<double, 3>& v, double dx, const std::vector<double>& geo_) const {
    auto distTo = [](const std::array<double, 3>& a, const std::array<double, 3>& b) {
        double sum = 0.0;
        for (int cc = 0; cc < 3; ++cc) sum += std::pow((a[cc] - b[cc]), 2);
        return std::sqrt(sum);
    };
    const std::array<double, 3> zero = {0.0, 0.0, 0.0};
    switch (shape) {
        case Shape::SPHERE: return !(distTo(v, loc) > geo_[0] + dx / 1.0e6);
        case Shape::HEMISPHERE: {
            if (distTo(v, loc) > geo_[0] + dx / 1.0e6) return false;
            return !(to_object(*this, v)[0] > dx / 1e6);
        }
        case Shape::BLOCK: {
            std::array<double, 3> t = to_object(*this, v);
            for (int i = 0; i < 3; ++i)
                if ((t[i] > geo_[i] / 2.0 + dx / 1.0e6) || (t[i] < -1.0 * geo_[i] / 2.0 - dx / 1.0e6)) return false;
            return true;
        }
        case Shape::ROUNDED_BLOCK: {
            std::array<double, 3> t = to_object(*this, v);
            const double rc = geo_.back();
            for (int i = 0; i < 3; ++i)
                if ((t[i] > geo_[i] / 2.0 + dx / 1.0e6) || (t[i] < -1.0 * geo_[i] / 2.0 - dx / 1.0e6)) return false;
            auto outer = [&](int i) { return (t[i] > geo_[i] / 2.0 - rc + dx / 1.0e6) || (t[i] < -1.0 * geo_[i] / 2.0 + rc - dx / 1.0e6); };
            auto inner = [&](int i) { return (t[i] < geo_[i] / 2.0 - rc + dx / 1.0e6) && (t[i] > -1.0 * geo_[i] / 2.0 + rc - dx / 1.0e6); };
            if (outer(0) || outer(1) || outer(2)) {
                for (int cc = 0; cc < 8; ++cc) {
                    const auto& c = curveCens[cc];
                    if ((std::sqrt(std::pow(t[0] - c[0], 2.0) + std::pow(t[1] - c[1], 2.0)) < rc + dx / 1.0e6) ||
                        (std::sqrt(std::pow(t[2] - c[2], 2.0) + std::pow(t[1] - c[1], 2.0)) < rc + dx / 1.0e6) ||
                        (std::sqrt(std::pow(t[0] - c[0], 2.0) + std::pow(t[2] - c[2], 2.0)) < rc + dx / 1.0e6))
                        return true;
                }
                if ((inner(0) && inner(1)) || (inner(2) && inner(1)) || (inner(0) && inner(2))) return true;
                return false;
            }
            return true;
        }
        case Shape::ELLIPSOID: {
            std::array<double, 3> t = to_object(*this, v);
            double ptSum = 0.0;
            for (int i = 0; i < (geo_[2] != 0.0 ? 3 : 2); ++i) ptSum += std::pow((t[i] - dx / 1.0e6) / (geo_[i] / 2.0), 2.0);
            if (1.0 < ptSum) return false;
            for (int i = 0; i < 3; ++i) {
                if ((2.0 * t[i] / geo_[i] < cutNeg[i]) || (2.0 * t[i] / geo_[i] > cutPos[i])) return false;
                if (cutGlobal[i] >= 0.0 && (t[i] + geo_[i] / 2.0) / geo_[i] >= cutGlobal[i]) return false;
                else if (cutGlobal[i] <= 0.0 && (t[i] - geo_[i] / 2.0) / geo_[i] <= cutGlobal[i]) return false;
            }
            return true;
        }
        case Shape::HEMIELLIPSOID: {
            std::array<double, 3> t = to_object(*this, v);
            if (t[0] > dx / 1e6) return false;
            double ptSum = 0.0;
            for (int i = 0; i < (geo_[2] != 0.0 ? 3 : 2); ++i) ptSum += std::pow((t[i] - dx / 1.0e6) / (geo_[i] / 2.0), 2.0);
            return !(1.0 < ptSum);
        }
        case Shape::CYLINDER: {
            std::array<double, 3> t = to_object(*this, v);
            if ((t[1] < -1.0 * geo_[1] / 2.0 - dx * 1e-6) || (t[1] > geo_[1] / 2.0 + dx * 1e-6)) return false;
            if (distTo({t[0], 0.0, t[2]}, zero) > geo_[0] + 1.0e-6 * dx) return false;
            return true;
        }
        case Shape::CONE: {
            std::array<double, 3> t = to_object(*this, v);
            if ((t[1] < -1.0 * geo_[1] / 2.0 - dx * 1e-6) || (t[1] > geo_[1] / 2.0 + dx * 1e-6)) return false;
            if (distTo({t[0], 0.0, t[2]}, zero) > std::pow(geo_[0] / geo_[2] * (t[2] - geo_[1] / 2.0), 2.0)) return false;
            return true;
        }
        case Shape::TRI_PRISM: {
            std::array<double, 3> t = to_object(*this, v);
            if ((t[2] < -1.0 * geo_[3] / 2.0 - dx * 1e-6) || (t[2] > geo_[3] / 2.0 + dx * 1e-6)) return false;
            const std::array<double, 3> b = to_bary<3>(invVert, t.data());
            for (int i = 0; i < 3; ++i)
                if (b[i] < -1e-13 || b[i] > geo_[i] + 1e-13) return false;
            if (std::abs(1 - (b[0] + b[1] + b[2])) > 1e-14) {
                baryFault->store(true);
                return false;
            }
            return true;
        }
        case Shape::TETRAHEDRON: {
            // The regular form keeps its two-entry size (side, height) as the emitter-buffer
            // geometry with which the material index is tested (geoParamML_ is copied before
            // the constructor replaces geoParam_, Obj.cpp:63-72 and 215-252), and the
            // reference reads four entries of it. No point passes that test in the
            // reference's runs (shapes_b, dip_surface_b); here it is false without the read.
            if (geo_.size() < 4) return false;
            const std::array<double, 4> b = to_bary<4>(invVert, v.data());
            for (int i = 0; i < 4; ++i)
                if (b[i] < -1e-6 * dx || (b[i] + dx * 1e-6) > geo_[i]) return false;
            if (std::abs(1 - (b[0] + b[1] + b[2] + b[3])) > 1e-14) {
                baryFault->store(true);
                return false;
            }
            return true;
        }
        case Shape::TERS_TIP: {
            std::array<double, 3> t = to_object(*this, v);
            if (distTo(t, radCen) < geo_[0] / 2.0) return true;
            if ((t[2] < geo_[0] - geo_[2] / 2.0 - dx * 1e-6) || (t[2] > geo_[1] / 2.0 + dx * 1e-6)) return false;
            if ((std::pow(t[0], 2.0) + std::pow(t[1], 2.0)) * std::pow(std::cos(geo_[0]), 2.0) - std::pow(t[2] * std::sin(geo_[0]), 2.0) >
                dx * 1e-6)
                return false;
            return true;
        }
        case Shape::PARABOLOID: {
            std::array<double, 3> t = to_object(*this, v);
            t[1] += geo_[2] / 2.0;
            if (t[1] > geo_[2]) return false;
            if (std::pow(t[0] / geo_[0], 2.0) + std::pow(t[2] / geo_[1], 2.0) > t[1]) return false;
            return true;
        }
        case Shape::TORUS: {
            std::array<double, 3> t = to_object(*this, v);
            if (std::pow(std::sqrt(std::pow(t[0], 2.0) + std::pow(t[1], 2.0)) - geo_[0], 2.0) > std::pow(geo_[1], 2.0) - std::pow(t[2], 2.0))
                return false;
            double phiPt = t[0] != 0 ? std::atan(t[1] / t[0]) : t[1] / std::abs(t[1]) * M_PI / 2.0;
            if (t[0] < 0) phiPt += M_PI;
            else if (t[1] < 0) phiPt += 2.0 * M_PI;
            if (phiPt < geo_[2] || phiPt > geo_[3]) return false;
            return true;
        }
    }
    return false;
}

// ---- surface directions (Obj::findGradient, OBJECTS/Obj.cpp:585-878) ----
namespace {

double sumSq(const std::array<double, 3>& v) { return ((0.0 + v[0] * v[0]) + v[1] * v[1]) + v[2] * v[2]; }

void normalize3(std::array<double, 3>& v) {
    const double n = std::sqrt(sumSq(v));
    for (auto& x : v) x = x / n;
}

// BLAS i?amin / i?amax: the first index (0-based here) of the smallest / largest |x|.
template <std::size_t N>
int first_abs_min(const std::array<double, N>& x) {
    int b = 0;
    for (int i = 1; i < static_cast<int>(N); ++i)
        if (std::abs(x[i]) < std::abs(x[b])) b = i;
    return b;
}
template <std::size_t N>
int first_abs_max(const std::array<double, N>& x) {
    int b = 0;
    for (int i = 1; i < static_cast<int>(N); ++i)
        if (std::abs(x[i]) > std::abs(x[b])) b = i;
    return b;
}

// Obj::ObjectSpace2RealSpace (Obj.cpp:24-34): the inverse of the unit-vector matrix (LU
// inverse, as the reference's constructor forms it) applied, then normalised (zero for a
// vector of squared length below 1e-20).
std::array<double, 3> to_real_normalised(const Object& o, const std::array<double, 3>& g) {
    double inv[9];
    std::copy(o.coord.begin(), o.coord.end(), inv);
    if (lu_invert(3, inv) == 0.0) throw InputError("The invCoordTransform_ can't be calculated!");
    std::array<double, 3> r;
    for (int i = 0; i < 3; ++i) {
        double t = 0.0;
        for (int k = 0; k < 3; ++k) t += inv[k + 3 * i] * g[k];
        r[i] = t;
    }
    if (sumSq(r) < 1e-20) return {0.0, 0.0, 0.0};
    normalize3(r);
    return r;
}

}  // namespace

std::array<double, 3> Object::gradient(const std::array<double, 3>& pt) const {
    const std::vector<double>& g = geo;
    switch (shape) {
        case Shape::SPHERE:
        case Shape::HEMISPHERE: {
            std::array<double, 3> r = {pt[0] - loc[0], pt[1] - loc[1], pt[2] - loc[2]};
            if (sumSq(r) < 1e-20) return {0.0, 0.0, 0.0};
            normalize3(r);
            return r;
        }
        case Shape::ELLIPSOID:
        case Shape::HEMIELLIPSOID: {
            std::array<double, 3> v = to_object(*this, pt);
            for (int i = 0; i < 3; ++i) v[i] = v[i] / std::pow(g[i], 2.0);
            return to_real_normalised(*this, v);
        }
        case Shape::CONE: {
            const std::array<double, 3> v = to_object(*this, pt);
            const double zp = v[2] + g[1] / 2.0;
            const double c = g[0] / g[2];
            const double z0 = zp * (1.0 + std::sqrt((std::pow(v[0], 2.0) + std::pow(v[1], 2.0)) / std::pow(c, 2.0)));
            std::array<double, 3> r = {2.0 * v[0], 2.0 * v[1], -2.0 * std::pow(c, 2.0) * (zp - z0)};
            if (std::abs(v[2]) == std::abs(z0 / 2.0)) r = {0.0, 0.0, -2.0 * v[2] / g[1]};
            return to_real_normalised(*this, r);
        }
        case Shape::CYLINDER: {
            const std::array<double, 3> v = to_object(*this, pt);
            const double r = std::sqrt(std::pow(v[0], 2.0) + std::pow(v[2], 2.0));
            const double len = g[1] * (r / g[0]);
            std::array<double, 3> d = {v[0], 0.0, v[2]};
            if (std::abs(v[1]) >= len / 2.0) d = {0.0, v[1] / std::abs(v[1]), 0.0};
            return to_real_normalised(*this, d);
        }
        case Shape::BLOCK:
        case Shape::ROUNDED_BLOCK: {
            const std::array<double, 3> v = to_object(*this, pt);
            std::array<double, 3> rat;
            for (int i = 0; i < 3; ++i) rat[i] = v[i] / g[i];
            const int m = first_abs_max(rat);
            std::array<double, 3> d = {0.0, 0.0, 0.0};
            bool corner = false;
            if (shape == Shape::ROUNDED_BLOCK) {
                const double t = rat[m];
                corner = true;
                for (int i = 0; i < 3; ++i)
                    if (v[i] - t * (g[i] - g[3]) <= 0) corner = false;
                if (corner) {
                    // the reference takes |pt| of the real-space point here
                    const std::array<double, 3> ab = {std::abs(pt[0]), std::abs(pt[1]), std::abs(pt[2])};
                    const std::array<double, 3>& cen = curveCens[0];
                    double dot = 0.0;
                    for (int k = 0; k < 3; ++k) dot += ab[k] * cen[k];
                    const double cenMag = sumSq(cen), ptMag = sumSq(ab);
                    const double tt = 1.0 / (cenMag - std::pow(g[3], 2.0)) *
                                      (std::pow(dot, 2.0) - std::sqrt(std::pow(dot, 2.0) - ptMag * (cenMag - std::pow(g[3], 2.0))));
                    for (int k = 0; k < 3; ++k) d[k] = ab[k] - tt * cen[k];
                    for (int k = 0; k < 3; ++k) d[k] = d[k] * pt[k] / std::abs(pt[k]);
                }
            }
            if (!corner)
                for (int i = 0; i < 3; ++i)
                    if (rat[i] == rat[m]) d[i] = v[i] >= 0 ? 1.0 : -1.0;
            return to_real_normalised(*this, d);
        }
        case Shape::TETRAHEDRON: {
            const std::array<double, 4> b = to_bary<4>(invVert, pt.data());
            std::array<double, 4> baseRat, truncRat;
            for (int i = 0; i < 4; ++i) {
                baseRat[i] = b[i] / g[i];
                truncRat[i] = (g[i] - b[i]) / g[i];
            }
            const int iB = first_abs_min(baseRat) + 1, iT = first_abs_min(truncRat) + 1;
            const int closest = (truncRat[iT - 1] < baseRat[iB - 1]) ? -1 * iT : iB;
            const double dist = (closest < 0) ? truncRat[iT - 1] : baseRat[iB - 1];
            std::vector<int> faces;
            for (int i = 0; i < 4; ++i) {
                if (baseRat[i] == dist) faces.push_back(i + 1);
                if (truncRat[i] == dist) faces.push_back(-1 * i - 1);
            }
            std::array<double, 3> d = {0.0, 0.0, 0.0};
            for (int f : faces) {
                // the face's vertices, ordered so that the cross product points outwards
                std::vector<int> act;
                const int af = std::abs(f);
                for (int ii = 0; ii < 4; ++ii) {
                    int index = (static_cast<int>(std::pow(-1, af - 1) * ii) % 4) * static_cast<int>(f / af);
                    index += (index < 0) ? 4 : 0;
                    if (index != af - 1) act.push_back(index);
                }
                std::array<double, 3> v1, v2;
                for (int k = 0; k < 3; ++k) {
                    v1[k] = verts[act[1]][k] - verts[act[0]][k];
                    v2[k] = verts[act[2]][k] - verts[act[1]][k];
                }
                std::array<double, 3> n = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
                normalize3(n);
                for (int k = 0; k < 3; ++k) d[k] = n[k] + d[k];
            }
            if (std::abs(sumSq(d)) < 1.0e-20) return {0.0, 0.0, 0.0};
            normalize3(d);
            return d;
        }
        case Shape::PARABOLOID: {
            std::array<double, 3> v = to_object(*this, pt);
            v[1] += g[2] / 2.0;
            std::array<double, 3> d = {2 * v[0] / std::pow(g[0], 2.0), -1.0, 2.0 * v[2] / std::pow(g[2], 2.0)};
            normalize3(d);
            return d;
        }
        case Shape::TORUS: {
            const std::array<double, 3> v = to_object(*this, pt);
            const double ring = std::sqrt(std::pow(v[0], 2.0) + std::pow(v[1], 2.0));
            const double term = (ring - g[0]) / ring;
            std::array<double, 3> d = {2.0 * v[0] * term, 2.0 * v[1] * term, 2.0 * v[2]};
            normalize3(d);
            return d;
        }
        case Shape::TERS_TIP:
            throw InputError("Gradient is not defined for this object yet defined");
        case Shape::TRI_PRISM:
            // tri_prism::findGradient (Obj.cpp:700-792) indexes its three vertices with a
            // 1-based face number, and with a negative one for the truncated faces, so its
            // result depends on memory past the vertex array
            throw UnsupportedError("dipoles relative to the surface of a triangular prism are not supported (the "
                                   "reference's prism gradient reads past its vertex array)");
    }
    return {0.0, 0.0, 0.0};
}

}  // namespace chiml
