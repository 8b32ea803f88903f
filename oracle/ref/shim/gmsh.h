// Declarations of the GMSH API calls FRICO makes. The definitions in
// ref_driver.cpp serve an in-memory triangle soup instead of meshing CAD.
#pragma once
#include <string>
#include <utility>
#include <vector>
namespace gmsh {
typedef std::vector<std::pair<int, int>> vectorpair;
void initialize(int argc = 0, char** argv = nullptr, bool readConfigFiles = true, bool run = false);
void finalize();
void clear();
void open(const std::string& fileName);
namespace option { void setNumber(const std::string& name, double value); }
namespace model {
void add(const std::string& name);
void getEntities(vectorpair& dimTags, int dim = -1);
void getPhysicalGroups(vectorpair& dimTags, int dim = -1);
void getPhysicalName(int dim, int tag, std::string& name);
void getEntitiesForPhysicalGroup(int dim, int tag, std::vector<int>& tags);
namespace mesh {
void getNodes(std::vector<std::size_t>& nodeTags, std::vector<double>& coord, std::vector<double>& parametricCoord,
              int dim = -1, int tag = -1, bool includeBoundary = false, bool returnParametricCoord = true);
void getElementTypes(std::vector<int>& elementTypes, int dim = -1, int tag = -1);
void getElementsByType(int elementType, std::vector<std::size_t>& elementTags, std::vector<std::size_t>& nodeTags,
                       int tag = -1, std::size_t task = 0, std::size_t numTasks = 1);
void generate(int dim = 3);
void setOrder(int order);
void setSize(const vectorpair& dimTags, double size);
}  // namespace mesh
namespace occ {
int addRectangle(double x, double y, double z, double dx, double dy, int tag = -1, double roundedRadius = 0.);
int addSphere(double xc, double yc, double zc, double radius, int tag = -1, double angle1 = -1.5707963267948966,
              double angle2 = 1.5707963267948966, double angle3 = 6.283185307179586);
void rotate(const vectorpair& dimTags, double x, double y, double z, double ax, double ay, double az, double angle);
void synchronize();
}  // namespace occ
}  // namespace model
}  // namespace gmsh
