/* Empty stand-in for lib/geometry/objects/_bbtree.hpp (included by
 * lib/geometry/objects/_objects.hpp:21, not shipped). Nothing on the
 * projection path uses it. */
