// Barnes-Hut node records as Solver::tree() hands them out: the 48-byte bh::Node layout of
// stett/nbody (include/nbody/bhtree.h), and a Tree that holds a node array. In this library
// the tree is built on the device; Tree::assign takes the exported node array
// (nbody_cuda_tree_export). Insertion, traversal and ray queries are the reference's own
// CPU octree (source/bhtree.cpp) and are not part of this library.
#pragma once
#include <cstdint>
#include <vector>
#include "nbody/vector.h"

namespace nbody
{
    struct Bounds
    {
        Vector center;
        float size = 0;
    };

    namespace bh
    {
        struct Node
        {
            Bounds bounds;
            Vector com;
            float mass = 0;
            uint32_t next = 0;      // next sibling, or the parent's next
            uint32_t children = 0;  // first of 8 contiguous children; 0 for a leaf
            uint32_t __pad0 = 0;
            uint32_t __pad1 = 0;
        };
        static_assert(sizeof(Node) == 48, "bh::Node must stay 48 bytes");

        class Tree
        {
        public:
            explicit Tree(const Bounds& bounds = { .center = {}, .size = 1 }) { clear(bounds); }

            void clear(const Bounds& bounds)
            {
                _nodes.assign(1, Node{});
                _nodes[0].bounds = bounds;
            }

            // Replace the nodes wholesale (root first).
            void assign(std::vector<Node> nodes) { _nodes = std::move(nodes); }

            [[nodiscard]] const Bounds& bounds() const { return _nodes[0].bounds; }
            [[nodiscard]] const std::vector<Node>& nodes() const { return _nodes; }

        private:
            std::vector<Node> _nodes;
        };
    }
}

// This header's Tree can take a node array wholesale (used by CudaSolver::tree()).
#define NBODY_TREE_ASSIGN 1
