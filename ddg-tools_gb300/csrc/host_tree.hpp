// Host-side (C++) parts of the Barnes-Hut / block-tree build: surface validation, FP64 face
// geometry and the face BVH. The BVH is built once per step; everything evaluated per
// energy or product runs on the device.
#pragma once
#include <array>
#include <cstdint>
#include <future>
#include <vector>

namespace rsg {

// Surface::new topology checks (RS/src/surface.rs:132-330).
void validate_topology(int nv, int nf, const uint32_t *faces);

// While alive on a thread, validate_topology on that thread returns at once: for a caller that
// validated the face list itself and rebuilds trees over it every step (the flow session,
// whose topology never changes).
struct TrustedTopology {
  TrustedTopology();
  ~TrustedTopology();
  TrustedTopology(const TrustedTopology &) = delete;
  TrustedTopology &operator=(const TrustedTopology &) = delete;
  bool prev;
};
// Whether this thread runs under a TrustedTopology (a worker thread takes its caller's trust
// over by making its own).
bool topology_trusted();
// Surface::validate_positions (RS/src/surface.rs:513-541).
void validate_positions(int nv, int nf, const uint32_t *faces, const double *pos);

// Face area, unit normal and barycenter in FP64, operation for operation as
// face_quantities (RS/src/geometry.rs:33-39), so that the tree matches the crate's.
struct FaceGeom {
  std::vector<double> area;   // F
  std::vector<double> normal; // 3F
  std::vector<double> bary;   // 3F
};
FaceGeom face_geometry(int nf, const uint32_t *faces, const double *pos);

// A BVH over points with boxes and masses (the generic Bvh<3> of
// RC/src/spatial/bvh.rs:114-290): nodes in pre-order, left child = i + 1, `right` = 0 for a
// leaf, node elements = order[start, end).
struct Tree {
  std::vector<uint32_t> start, end, right, order;
  std::vector<double> box;       // 6 per node: lo xyz, hi xyz (build positions)
  std::vector<double> mass;      // per node
  std::vector<double> centroid;  // 3 per node
  std::vector<double> radius;    // farthest box corner from the centroid (spatial/mod.rs:143-150)
  std::vector<uint32_t> leaves;  // node ids of the leaves, increasing
  std::vector<uint32_t> leaf_ordinal;  // per node: its index in `leaves` or UINT32_MAX
  size_t n_nodes() const { return start.size(); }
};

// Builds the tree over `n` elements with points `pts` (3n), element boxes `ebox` (6n: lo, hi)
// and masses `mass` (n), leaf size `leaf_size`, balance floor 1/4 (bvh.rs:126-220), and its
// node data as Bvh::refit computes it (bvh.rs:226-260).
Tree build_tree(size_t n, const double *pts, const double *ebox, const double *mass,
                int leaf_size);

// The face elements of FaceTree (RS/src/spatial/mod.rs:56-76): barycenter, box of the three
// vertices, area.
Tree build_face_tree(int nf, const uint32_t *faces, const double *pos, const FaceGeom &g,
                     int leaf_size);

// A face geometry and face tree built once and offered, on the threads that hold one of these,
// to the builders that would build the same ones: the flow step builds its BVH once for the
// Barnes-Hut lists and the metric's block cluster tree. A builder asks with its faces and
// positions (the same arrays, compared by address), face count and leaf size.
struct SharedFaceTree {
  // ready (optional): completed when geom and tree are built; a lookup waits for it and
  // rethrows the builder's exception
  SharedFaceTree(const FaceGeom &g, const Tree &t, const uint32_t *faces, const double *pos, int nf,
                 int leaf_size, const std::shared_future<void> *ready);
  ~SharedFaceTree();
  SharedFaceTree(const SharedFaceTree &) = delete;
  SharedFaceTree &operator=(const SharedFaceTree &) = delete;
  const FaceGeom &geom;
  const Tree &tree;
  const uint32_t *faces;
  const double *pos;
  int nf, leaf_size;
  const std::shared_future<void> *ready;
  const SharedFaceTree *prev;
};
// The shared tree on this thread for these arguments, or null.
const SharedFaceTree *shared_face_tree(const uint32_t *faces, const double *pos, int nf, int leaf_size);

}  // namespace rsg
