/*
 * The reference's dynamic-walk example (src/examples/dynamic_walk.cpp:30-93)
 * on this engine's C++ classes (walk_engine.cuh).
 *
 * The program is the reference's, line for line, with its includes changed
 * and its lambdas turned into __device__ functors: a weighted first-order
 * walk whose dynamic component doubles the edge back to the vertex the walker
 * came from (1 at step 0, 2 for the return edge, 1 otherwise, upper bound 2),
 * the walker state remembering that vertex (UINT_MAX before the first step).
 *
 * Options follow the reference's TruncatedRandomWalkOptionHelper
 * (include/option_helper.hpp:106-181): -v vertex count, -g graph file
 * (binary Edge<real_t> records), --make-undirected, -o output prefix, -r rate,
 * -l walk length (default 80), -w walker count (the reference example fixes
 * it at 34, the default here); --seed sets the walk's Philox key (default 1).
 *
 * Built into knightking_gb300/lib/libkk_example_dynamic_walk.so; the entry
 * point kk_example_dynamic_walk(argc, argv) is the program's main.
 */
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>

#include "knightking_gb300/walk_engine.cuh"

using namespace kk;

namespace
{

struct WalkState
{
    vertex_id_t last_vertex;
};

struct InitWalker
{
    __device__ void operator()(Walker<WalkState> &walker, vertex_id_t start_vertex, Sampler &) const
    {
        /*At first, the last vertex is not defined*/
        walker.data.last_vertex = UINT_MAX;
    }
};

struct UpdateWalker
{
    __device__ void operator()(Walker<WalkState> &walker, vertex_id_t current_v, const AdjUnit &edge) const
    {
        walker.data.last_vertex = current_v;
    }
};

struct ExtensionComp
{
    step_t walk_length;
    __device__ real_t operator()(const Walker<WalkState> &walker, vertex_id_t current_v) const
    {
        return walker.step >= walk_length ? 0.0 : 1.0; /*walk walk_length steps then terminate*/
    }
};

struct StaticComp
{
    const real_t *weight; /* the edge data the reference reads as edge->data */
    __device__ real_t operator()(vertex_id_t v, const AdjUnit &edge) const
    {
        return weight[edge.index]; /*edge->data is a real number denoting edge weight*/
    }
};

struct DynamicComp
{
    __device__ real_t operator()(const Walker<WalkState> &walker, vertex_id_t current_v, const AdjUnit &edge) const
    {
        if (walker.step == 0)
        {
            /*No return edge for the first step*/
            return 1.0;
        }
        else if (edge.neighbour == walker.data.last_vertex)
        {
            /*if return edge, double the un-normalized transition probability*/
            return 2.0;
        }
        else
        {
            /*if not return edge*/
            return 1.0;
        }
    }
};

struct DynamicCompUpperbound
{
    __device__ real_t operator()(vertex_id_t v_id, const AdjList &adj_lists) const { return 2.0; }
};

struct Options
{
    vertex_id_t v_num = 0;
    std::string graph_path, output_path;
    bool make_undirected = false, set_rate = false;
    double rate = 1.0;
    step_t walk_length = 80;
    walker_id_t walker_num = 34;
    uint64_t seed = 1;
};

bool parse(int argc, char **argv, Options &opt)
{
    for (int i = 1; i < argc; i++)
    {
        const std::string k = argv[i];
        const bool has = i + 1 < argc;
        if (k == "--make-undirected")
            opt.make_undirected = true;
        else if (k == "-v" && has)
            opt.v_num = (vertex_id_t)strtoul(argv[++i], nullptr, 10);
        else if (k == "-g" && has)
            opt.graph_path = argv[++i];
        else if (k == "-o" && has)
            opt.output_path = argv[++i];
        else if (k == "-r" && has)
        {
            opt.rate = strtod(argv[++i], nullptr);
            opt.set_rate = true;
        }
        else if (k == "-l" && has)
            opt.walk_length = (step_t)strtoul(argv[++i], nullptr, 10);
        else if (k == "-w" && has)
            opt.walker_num = (walker_id_t)strtoul(argv[++i], nullptr, 10);
        else if (k == "--seed" && has)
            opt.seed = strtoull(argv[++i], nullptr, 10);
        else
            return false;
    }
    return opt.v_num > 0 && !opt.graph_path.empty();
}

} // namespace

extern "C" int kk_example_dynamic_walk(int argc, char **argv)
{
    Options opt;
    if (!parse(argc, argv, opt))
    {
        fprintf(stderr, "usage: dynamic_walk -v V -g graph [--make-undirected] [-o out] [-r rate] [-l length] "
                        "[-w walkers] [--seed s]\n");
        return 2;
    }
    try
    {
        WalkEngine<real_t, WalkState> graph;
        graph.load_graph(opt.v_num, opt.graph_path.c_str(), opt.make_undirected);
        graph.set_seed(opt.seed);
        WalkConfig walk_conf;
        if (!opt.output_path.empty())
        {
            walk_conf.set_output_file(opt.output_path.c_str());
        }
        if (opt.set_rate)
        {
            walk_conf.set_walk_rate(opt.rate);
        }

        auto walker_conf = make_walker_config<WalkState>(opt.walker_num, InitWalker{}, UpdateWalker{});
        auto tr_conf = make_transition_config<WalkState>(ExtensionComp{opt.walk_length},
                                                         StaticComp{graph.edge_weights()}, DynamicComp{},
                                                         DynamicCompUpperbound{});
        graph.random_walk(&walker_conf, &tr_conf, &walk_conf);
    }
    catch (const Error &err)
    {
        fprintf(stderr, "dynamic_walk: %s (status %d)\n", err.msg.c_str(), (int)err.status);
        return 1;
    }
    return 0;
}
