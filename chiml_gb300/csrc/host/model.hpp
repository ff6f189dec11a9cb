// Input model of a chiML simulation: the parsed JSON input, in FDTD units.
//
// Field names follow chiML's parallelProgramInputs (INPUTS/parallelInputs.hpp)
// so that each value can be traced to the line of parallelInputs.cpp that
// produces it. Only the features of the time-step loop handled by this
// library are representable; everything else is rejected at parse time with
// UnsupportedError (there is no CPU fallback).
#pragma once

#include <array>
#include <atomic>
#include <cmath>
#include <complex>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "json.hpp"

namespace chiml {

typedef std::complex<double> cplx;

struct UnsupportedError : public std::runtime_error {
    explicit UnsupportedError(const std::string& w) : std::runtime_error(w) {}
};

// Physical constants exactly as UTIL/ml_consts.hpp:13-17 defines them.
extern const double kSpeedOfLight;
extern const double kEps0;
extern const double kElementaryCharge;
extern const double kHbar;

enum class Pol { EX, EY, EZ, HX, HY, HZ, L, R };
enum class PulseShape { GAUSSIAN, CONTINUOUS, RICKER, RAMP_CONT, BH, RECT };
// OBJECTS/Obj.hpp:491-1290 (TRI_PRISM covers the reference's triangle and trapezoid prisms)
enum class Shape {
    SPHERE,
    BLOCK,
    ELLIPSOID,
    CYLINDER,
    HEMISPHERE,
    ROUNDED_BLOCK,
    HEMIELLIPSOID,
    CONE,
    TRI_PRISM,
    TERS_TIP,
    PARABOLOID,
    TORUS,
    TETRAHEDRON
};
enum class DipOr { REL_TO_NORM, ISOTROPIC, UNIDIRECTIONAL, LONG_TAN, LAT_TAN };
enum class DtcClass { TXT, BIN, FREQ };
// Same ordering as DTCTYPE (UTIL/enum.hpp:17)
enum class DtcType { EX, EY, EZ, HX, HY, HZ, DX, DY, DZ, BX, BY, BZ, EPOW, HPOW, PX, PY, PZ };

// One Lorentz oscillator of a custom material (LorenzDipoleOscillator, OBJECTS/Obj.hpp:18-39).
struct Oscillator {
    DipOr dipOrE = DipOr::ISOTROPIC;
    double omg = 0.0, gam = 0.0, sigP = 0.0;
    std::array<double, 3> uVecDipE = {1.0, 1.0, 1.0};
    // weights of a dipole relative to the local surface (normCompWeightE_,
    // tangentLatCompWeightE_, tangentLongCompWeightE_; parallelInputs.cpp:1330-1357)
    double normW = 1.0, latW = 0.0, longW = 0.0;
};

// A geometric object with its material; coefficients from Obj::setUpConsts (Obj.cpp:299-370).
struct Object {
    Shape shape = Shape::BLOCK;
    bool ML = false;               // has an emitter basis set
    double epsInf = 1.0;
    double muInf = 1.0;            // constant relative permeability (no magnetic poles)
    std::vector<double> geo;       // shape parameters (Obj::geoParam_)
    std::vector<double> geoML;     // geoParamML_: geo with the emitter buffer added
    std::array<double, 3> loc = {0.0, 0.0, 0.0};
    std::array<double, 9> coord = {1, 0, 0, 0, 1, 0, 0, 0, 1};  // rows: normalised unit vectors
    std::array<double, 3> cutNeg = {-1, -1, -1}, cutPos = {1, 1, 1}, cutGlobal = {1, 1, 1};
    // shape data built from geo when the object is read (Obj.cpp:133-272)
    std::array<std::array<double, 3>, 8> curveCens{};  // rounded block: corner centres of curvature
    std::array<std::array<double, 3>, 4> verts{};      // prism: 2-D vertices about the centroid; tetrahedron: 3-D vertices
    std::array<double, 16> invVert{};                  // inverse of the vertex matrix (column-major, order 3 or 4)
    std::array<double, 3> radCen{};                    // TERS tip: centre of the apex sphere
    // Set when a barycentric test of a prism or tetrahedron fails its sum check (the
    // reference throws there); shared by the copies of the object.
    std::shared_ptr<std::atomic<bool>> baryFault = std::make_shared<std::atomic<bool>>(false);
    std::vector<Oscillator> pols;
    // derived per time step (setUpConsts)
    bool orDip = false;
    std::vector<double> alpha, xi, gamma;
    std::vector<double> alphaInc;  // -(omega dt)^2 / (1 + gamma dt) = alpha + xi - 1, formed without cancellation
    std::vector<DipOr> dipOr;
    std::vector<std::array<double, 3>> dipE;
    std::vector<std::array<double, 3>> dipW;  // per pole: normal, latitudinal, longitudinal weights

    bool isObj(const std::array<double, 3>& v, double dx, const std::vector<double>& g) const;
    // Outward surface direction at a real-space point (Obj::findGradient, Obj.cpp:585-878).
    std::array<double, 3> gradient(const std::array<double, 3>& pt) const;
    bool isVacuum() const { return !(gamma.size() > 0 || epsInf != 1.0 || ML); }
    void setUpConsts(double dt);
};

struct PulseSpec {
    PulseShape shape = PulseShape::GAUSSIAN;
    std::vector<cplx> param;  // parameter list as built in parallelInputs.cpp:133-172 (+ amplitude appended)
    cplx value(double t) const;
};

struct SourceSpec {
    Pol pol = Pol::EZ;
    std::vector<PulseSpec> pulses;
    std::array<int, 3> loc = {0, 0, 0}, sz = {1, 1, 1};
    double phi = 90.0;
};

// A TFSF plane-wave surface (parallelInputs.cpp:219-408): box in grid points (lower
// corner, 0-based physical coordinates, and size), integer propagation vector m, angles
// in radians, pulses (amplitude appended as (0, Emax)), polarisation and the 1-D CPML.
struct TfsfSpec {
    std::array<int, 3> loc = {0, 0, 0}, sz = {1, 1, 1}, m = {0, 0, 0};
    double theta = M_PI / 2.0, phi = 0.0, psi = 0.0;
    std::vector<PulseSpec> pulses;
    Pol circPol = Pol::EX;
    double kRatio = 1.0;
    int pmlThick = 20;
    double pmlAMax = 0.0, pmlM = 3.0, pmlMa = 1.0;
};

struct DetectorSpec {
    DtcClass cls = DtcClass::TXT;
    DtcType type = DtcType::EZ;
    std::string name;
    std::array<int, 3> loc = {0, 0, 0}, sz = {1, 1, 1};
    bool SI = true;
    double timeInt = 0.0;
    std::vector<double> freqList;
    bool outputMaps = false;
};

struct FluxSpec {
    std::string name;
    std::array<int, 3> loc = {0, 0, 0}, sz = {1, 1, 1};
    double weight = 1.0;
    int timeInt = 1;
    std::vector<double> freqList;
    bool SI = false, crossSec = false, save = false, load = false;
    std::string incdFile;
};

// One energy-level descriptor of the emitters (EnergyLevelDiscriptor; built in
// parallelInputs.cpp:465-579): the energies it can take (FDTD units), their weights,
// and how many basis levels it describes.
struct EnergyLevel {
    std::vector<double> energyStates;
    std::vector<double> weights;
    int levDescribed = 1;
};

// One relaxation channel of an emitter (relaxParams, ML/parallelQE.hpp:22-28); rates in FDTD units.
struct RelaxOp {
    int n0 = 0, nf = 0;
    double rate = 0.0, dephasing = 0.0;
};

// A quantum-emitter object (parallelInputs.cpp:453-660): the object index, its
// (l, m) basis, molecular density, transition-dipole couplings (FDTD units), the
// relaxation matrix or channels, the grid points it holds, and its outputs.
struct EmitterSpec {
    int object = -1;
    std::vector<std::array<int, 2>> basis;
    double molDen = 1.0;
    std::vector<double> couplings;
    std::vector<std::vector<double>> gam;  // given relaxation matrix (may be empty)
    std::vector<RelaxOp> relax;
    std::vector<std::array<int, 3>> locs;  // physical grid points, z outermost then y then x
    bool outputPol = false;
    std::string polFile;
    std::vector<int> dtcLevs;
    std::vector<std::string> dtcFiles;
    int dtcTimeInt = 1;
    // Extension (no reference counterpart; the reference reads none of these keys): a
    // per-cell dipole for an object whose operator lies along z. "dipole_orientation":
    // "random" turns each cell's dipole to a direction drawn uniformly on the sphere,
    // "z" keeps it along z; "dipole_scale_range" [a, b] scales each cell's operator by a
    // factor drawn uniformly from [a, b); both from a PCG32 stream seeded by "dipole_seed".
    bool cellDipole = false;
    bool randomDirection = false;
    std::array<double, 2> dipoleScale = {1.0, 1.0};
    unsigned long long dipoleSeed = 0;
};

struct Inputs {
    std::string filename;
    Pol pol = Pol::EZ;
    double a = 1e-7, I0 = 0.0, tMax = 0.0, courant = 0.5, dt = 0.0;
    int res = -1;
    std::array<double, 3> size = {0, 0, 0}, d = {0, 0, 0};
    // PML
    std::array<int, 3> pmlThickness = {0, 0, 0};
    double pmlSigOptRat = 1.0, pmlKappaMax = 1.0, pmlAMax = 0.0, pmlMa = 1.0, pmlM = 3.0;
    std::vector<SourceSpec> sources;
    std::vector<TfsfSpec> tfsf;
    std::vector<Object> objects;  // objects[0] is the vacuum cell block
    std::vector<DetectorSpec> detectors;
    std::vector<FluxSpec> fluxes;
    // energy-level descriptors of all emitters together (the reference keeps one list, qeELevs_)
    std::vector<EnergyLevel> qeELevs;
    std::vector<EmitterSpec> emitters;

    int nSteps() const;
};

// Builds Inputs from a parsed JSON tree (parallelProgramInputs ctor, parallelInputs.cpp:12-838).
Inputs read_inputs(const JNode& root, const std::string& filename);
Inputs read_inputs_file(const std::string& path);

}  // namespace chiml
