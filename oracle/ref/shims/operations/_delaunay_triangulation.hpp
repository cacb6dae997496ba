/* Empty stand-in for lib/geometry/operations/_delaunay_triangulation.hpp
 * (included by lib/geometry/geometry.hpp:18, not shipped). Nothing on the
 * projection path uses it. */
