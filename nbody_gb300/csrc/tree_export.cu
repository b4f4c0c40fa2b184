// The last device tree in the reference's own node layout, for Solver::tree() / Sim::nodes()
// (include/nbody/bhtree.h:13-22): 48-byte nodes {bounds centre, size, com, mass, next,
// children, pad, pad}; a split node owns 8 contiguous children, child q at children + q
// where q is the reference octant (bit set when the coordinate is below the centre,
// bounds.h:31-38); child q's `next` is the next sibling and child 7's is the parent's
// `next`, so the stackless walk of bhtree.cpp:97-138 runs over it unchanged.
//
// The device tree keeps only the cells the traversal needs. Expanding it back:
//   - a cell whose bodies all sit in one octant of the cell above is, in the reference, a
//     chain of single-child cells with the same mass and centre of mass: emitted as such;
//   - octants holding nothing become the reference's empty leaves (mass 0);
//   - a single body becomes a leaf carrying its position and mass;
//   - bodies sharing one finest (level-21) Morton cell, which the reference would keep
//     subdividing down to FLT_EPSILON-sized cells (bhtree.cpp:36-42), become one leaf with
//     their total mass and centre of mass.
// Node order is depth-first (the reference's is insertion order); the links, cells, masses
// and centres of mass describe the same tree.
#include <cstring>
#include <vector>

#include "bh.cuh"
#include "context.cuh"

namespace nbg
{
    namespace
    {
        struct RefNode
        {
            float cx, cy, cz, size;
            float comx, comy, comz, mass;
            uint32_t next, children, pad0, pad1;
        };
        static_assert(sizeof(RefNode) == 48, "reference node layout");

        constexpr int kLevels = 21;

        struct Content
        {
            enum Kind { Empty, Body, Cell } kind = Empty;
            int index = 0;
        };

        class Exporter
        {
        public:
            explicit Exporter(const TreeSnapshot& t) : _t(t) {}

            std::vector<RefNode> run()
            {
                _out.clear();
                _out.reserve(_t.cells.size() * 9 + 16);
                _out.push_back(RefNode{});
                Content root;
                if (_t.n == 1)
                    root = { Content::Body, 0 };
                else if (_t.n >= 2)
                    root = { Content::Cell, 0 };
                fill(0, 0, 0, root);
                _out[0].next = 0;
                return _out;
            }

        private:
            static uint64_t compact1by2(uint64_t v)
            {
                v &= 0x1249249249249249ull;
                v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
                v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
                v = (v ^ (v >> 8)) & 0x001f0000ff0000ffull;
                v = (v ^ (v >> 16)) & 0x001f00000000ffffull;
                v = (v ^ (v >> 32)) & 0x1fffffull;
                return v;
            }

            // Level of a cell: the common prefix of its first and last codes, in octal digits.
            int cell_level(const OctNode& c) const
            {
                const uint64_t a = _t.codes[c.first], b = _t.codes[c.last];
                if (a == b)
                    return kLevels;
                const int prefix = __builtin_clzll(a ^ b) - 1;
                return prefix / 3 < kLevels ? prefix / 3 : kLevels;
            }

            static unsigned digit(const uint64_t code, const int level)   // octant at `level` (1..21)
            {
                return static_cast<unsigned>((code >> (3 * (kLevels - level))) & 7u);
            }

            void set_bounds(RefNode& nd, const int level, const uint64_t prefix) const
            {
                const double cell = _t.box.edge / static_cast<double>(1ull << level);
                const uint64_t ix = compact1by2(prefix), iy = compact1by2(prefix >> 1), iz = compact1by2(prefix >> 2);
                nd.cx = static_cast<float>(_t.box.lo[0] + (static_cast<double>(ix) + 0.5) * cell);
                nd.cy = static_cast<float>(_t.box.lo[1] + (static_cast<double>(iy) + 0.5) * cell);
                nd.cz = static_cast<float>(_t.box.lo[2] + (static_cast<double>(iz) + 0.5) * cell);
                nd.size = static_cast<float>(cell);
            }

            uint64_t code_of(const Content& c) const
            {
                return c.kind == Content::Body ? _t.codes[c.index] : _t.codes[_t.cells[c.index].first];
            }

            // Emit the reference node at `at` for the level-`level` cell `prefix` holding `c`.
            void fill(const uint32_t at, const int level, const uint64_t prefix, const Content c)
            {
                set_bounds(_out[at], level, prefix);
                _out[at].children = 0;
                if (c.kind == Content::Empty)
                {
                    _out[at].mass = 0.f;
                    _out[at].comx = _out[at].comy = _out[at].comz = 0.f;
                    return;
                }
                if (c.kind == Content::Body)
                {
                    const float4 b = _t.bodies[c.index];
                    _out[at].comx = b.x;
                    _out[at].comy = b.y;
                    _out[at].comz = b.z;
                    _out[at].mass = b.w;
                    return;
                }
                const OctNode& cell = _t.cells[c.index];
                _out[at].comx = cell.com_mass.x;
                _out[at].comy = cell.com_mass.y;
                _out[at].comz = cell.com_mass.z;
                _out[at].mass = cell.com_mass.w;
                const int lc = cell_level(cell);
                if (level >= kLevels || (cell.nchild < 0 && level >= lc))
                    return;         // finest cell: its bodies merge into this leaf

                Content slot[8];
                if (lc > level || cell.nchild < 0)
                {
                    // a reference chain cell: every body of `cell` in one octant
                    const unsigned d = digit(_t.codes[cell.first], level + 1);
                    slot[d ^ 7u] = c;
                }
                else
                {
                    for (int k = 0; k < cell.nchild; ++k)
                    {
                        const int ch = cell.child[k];
                        const Content cc = ch < 0 ? Content{ Content::Body, ~ch } : Content{ Content::Cell, ch };
                        slot[digit(code_of(cc), level + 1) ^ 7u] = cc;
                    }
                }
                const uint32_t block = static_cast<uint32_t>(_out.size());
                _out[at].children = block;
                const uint32_t parent_next = _out[at].next;
                for (unsigned q = 0; q < 8; ++q)
                {
                    RefNode child{};
                    child.next = q < 7 ? block + q + 1 : parent_next;
                    _out.push_back(child);
                }
                for (unsigned q = 0; q < 8; ++q)
                {
                    const unsigned d = q ^ 7u;
                    fill(block + q, level + 1, (prefix << 3) | d, slot[q]);
                }
            }

            const TreeSnapshot& _t;
            std::vector<RefNode> _out;
        };
    }
}

extern "C" int nbody_cuda_tree_export(nbody_cuda* ctx, void* nodes, const size_t max_nodes, size_t* count)
{
    using namespace nbg;
    if (!ctx || !count)
        return NBODY_ERR_INVALID;
    if (ctx->tree_export_id == 0 || ctx->tree_export_id != bh_build_id(ctx))
    {
        TreeSnapshot snap;
        if (const int st = bh_download(ctx, &snap))
            return st;
        const std::vector<RefNode> out = Exporter(snap).run();
        ctx->tree_export.resize(out.size() * sizeof(RefNode));
        std::memcpy(ctx->tree_export.data(), out.data(), ctx->tree_export.size());
        ctx->tree_export_id = snap.build_id;
    }
    const size_t have = ctx->tree_export.size() / sizeof(RefNode);
    *count = have;
    if (nodes && max_nodes)
        std::memcpy(nodes, ctx->tree_export.data(), (have < max_nodes ? have : max_nodes) * sizeof(RefNode));
    return NBODY_OK;
}
