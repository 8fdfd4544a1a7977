// Parameter model of a MITHRA job (host side), mirroring the parsed classes of the reference:
// Mesh, BunchInitialize/Bunch, Signal, Seed, Undulator, ExtField, FreeElectronLaser
// (src/classes.h:20-576, src/database.h:19-100).  Field names follow the job-file keys.
#pragma once
#include <array>
#include <cmath>
#include <string>
#include <vector>

namespace mithra {
namespace host {

using Vec3 = std::array<double, 3>;

// Constants of src/stdinclude.h:43-52.
constexpr double PI = 3.1415926535;
constexpr double EPSILON_ZERO = 8.85418782e-12;
constexpr double MU_ZERO = 4.0 * PI * 1.0e-7;
inline double C0() { return 1.0 / std::sqrt(EPSILON_ZERO * MU_ZERO); }
constexpr double EC = 1.602e-19;
constexpr double EM = 9.109e-31;

enum SignalType { NEUMANN, GAUSSIAN, SECANT, FLATTOP, INVGAUSSIAN };
enum SeedType { PLANEWAVE, PLANEWAVETRUNCATED, GAUSSIANBEAM, SUPERGAUSSIANBEAM, STANDINGPLANEWAVE,
                STANDINGPLANEWAVETRUNCATED, STANDINGGAUSSIANBEAM, STANDINGSUPERGAUSSIANBEAM };
enum UndulatorType { STATIC, OPTICAL };
enum SamplingType { ATPOINT, OVERLINE, INPLANE, ALLDOMAIN };
enum SolverType { FD, NSFD };

struct Signal {  // src/classes.cpp:500-575
  SignalType type = GAUSSIAN;
  double t0 = 0.0, s = 0.0, f0 = 1.0, cep = 0.0;
  unsigned nR = 1;
  std::vector<double> sigmaInvG = {0.0, 0.0};
  double self(double t, double phase) const;
};

struct Mesh {  // src/classes.h Mesh; defaults of Mesh::initialize (src/classes.cpp:38-46)
  double lengthScale = 0.0, timeScale = 0.0;
  Vec3 meshLength{0, 0, 0}, meshResolution{0, 0, 0}, meshCenter{0, 0, 0};
  double totalTime = 0.0, totalDist = 0.0, timeShift = 0.0, gamma = -1.0, timeStep = 0.0;
  int truncationOrder = 0;
  bool spaceCharge = false, optimizePosition = false;
  SolverType solver = NSFD;
};

struct BunchInit {  // src/database.h:19-100, defaults src/database.cpp:15-36
  std::string type, distribution, generator;
  unsigned numberOfParticles = 0;
  double cloudCharge = 0.0, initialGamma = 0.0, initialBeta = 0.0;
  Vec3 initialDirection{0, 0, 0};
  std::vector<Vec3> position;
  std::array<unsigned, 3> numbers{0, 0, 0};
  Vec3 latticeConstants{0, 0, 0}, sigmaPosition{0, 0, 0}, sigmaGammaBeta{0, 0, 0};
  double tranTrun = 0.0, longTrun = 0.0;
  std::string fileName;
  double lambda = 0.0, bF = 0.0, bFP = 0.0;
  bool shotNoise = false;
  Vec3 betaVector{0, 0, 0};
};

struct Bunch {
  std::vector<BunchInit> inits;
  double timeStep = 0.0;
  // bunch-sampling and bunch-profile (written by FdTd.solve); bunch-visualization is parsed for
  // compatibility and not produced.
  bool sampling = false, vtk = false, profile = false;
  double rhythm = 0.0, vtkRhythm = 0.0, profileRhythm = 0.0;
  std::string directory, basename;  // bunch-sampling file
  std::string profileDirectory, profileBasename;  // bunch-profile files
  std::vector<double> profileTime;
  double zu = 0.0, beta = 0.0;
};

// Shared by Seed, Undulator (optical) and ExtField: the laser-beam description.
struct Beam {
  SeedType seedType = PLANEWAVE;
  Vec3 position{0, 0, 0}, direction{0, 0, 0}, polarization{0, 0, 0};
  double amplitude = 0.0, a0 = 0.0;
  std::vector<double> radius = {0.0, 0.0};
  std::vector<int> order = {0, 0};
  Signal signal;
  double l = 0.0, c0 = 0.0;
  std::vector<double> zR = {0.0, 0.0};
};

// Seed::vtk (src/classes.h:216-229, defaults src/classes.cpp:858-868): one field-visualization
// output.  field codes: 0..9 = Ex Ey Ez Bx By Bz Ax Ay Az F (Seed::fieldType, src/classes.cpp:896-909).
enum VtkType { VTK_ALLDOMAIN = 0, VTK_INPLANE = 1 };
enum VtkPlane { VTK_XNORMAL = 0, VTK_YNORMAL = 1, VTK_ZNORMAL = 2 };
struct FieldVtk {
  bool sample = false;
  std::vector<int> field;
  std::string directory, basename;
  VtkType type = VTK_ALLDOMAIN;
  VtkPlane plane = VTK_ZNORMAL;
  double rhythm = 0.0;
  Vec3 position{0, 0, 0};
};

// field-sampling group (src/datainput.cpp:331-366): E, B, A at points or along a line.
struct FieldSampling {
  SamplingType type = ATPOINT;
  std::vector<int> field;  // codes as FieldVtk
  std::string directory, basename;
  double rhythm = 0.0;
  std::vector<Vec3> position;
  Vec3 lineBegin{0, 0, 0}, lineEnd{0, 0, 0};
  int res = 0;
};

struct Seed : Beam {  // src/classes.h Seed
  double beta = 0.0, gamma = 1.0, dt = 0.0;
  bool sampling = false, profile = false;
  FieldSampling samp;
  std::vector<FieldVtk> vtk;
  // Seed::fields (src/classes.cpp:740-855): the vector potential of the seed at a bunch-frame
  // point and time.  `a` is accumulated into for super-Gaussian beams, as in the reference.
  void fields(const Vec3& r, double time, Vec3& a) const;
};

struct Undulator : Beam {  // src/classes.h Undulator, defaults src/classes.cpp:973-996
  UndulatorType type = STATIC;
  double k = 0.0, lu = 0.0, rb = 0.0, dist = 0.0, theta = 0.0;
  unsigned length = 0;
};

struct ExtField : Beam {};

struct RadiationPower {  // FreeElectronLaser::RadiationSampling, src/classes.cpp:1300-1311
  bool sampling = false;
  std::vector<double> z;
  std::string directory, basename;
  double lineBegin = 0.0, lineEnd = 0.0;
  unsigned res = 0;
  SamplingType samplingType = ATPOINT;
  std::vector<double> lambda;
  double lambdaMin = 0.0, lambdaMax = 0.0;
  unsigned lambdaRes = 0;
};

struct ScreenProfile {  // FreeElectronLaser::ScreenProfile, src/classes.h:554-572, src/classes.cpp:1324-1331
  bool sampling = false;
  std::string directory = "./", basename;
  std::vector<double> pos;  // lab z of the screens, from the undulator start
  double rhythm = 0.0;
};

struct FEL {
  RadiationPower radiationPower;
  ScreenProfile screenProfile;
};

struct Job {
  Mesh mesh;
  Bunch bunch;
  Seed seed;
  std::vector<Undulator> undulators;
  std::vector<ExtField> extFields;
  std::vector<FEL> fel;
};

// Reads and parses a job file with the semantics of read_file/cleanJobFile
// (src/readdata.cpp:10-53) and ParseDarius (src/datainput.cpp:18-751).  Throws std::runtime_error
// with the reference's message where the reference would exit(1).
Job parse_job_file(const std::string& path);
Job parse_job_text(const std::vector<std::string>& lines);

}  // namespace host
}  // namespace mithra
