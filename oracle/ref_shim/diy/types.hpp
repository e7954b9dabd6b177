// Single-process stand-in for the DIY block-parallel library
// (github.com/diatomic/diy, header-only, not vendored by the reference).
// Test infrastructure only: it lets the reference's src/tet.cpp,
// src/volume.cpp and src/dense.cpp compile unmodified so that their outputs
// can pin the oracle.  Only the members those files and include/tess/*.hpp
// touch are provided.  Every block lives in this one process; enqueue/
// exchange/dequeue move bytes between per-block queues; in() reports the
// neighbours whose core bounds contain a point, boundaries inclusive (the
// behaviour of DIY's pick.hpp in(), restated).
#ifndef TESS_ORACLE_SHIM_DIY_TYPES_HPP
#define TESS_ORACLE_SHIM_DIY_TYPES_HPP

#include <vector>
#include <map>
#include <functional>
#include <cstring>
#include <cstddef>
#include "mpi.h"

namespace diy
{
    struct ContinuousBounds
    {
        float min[4];
        float max[4];
        ContinuousBounds(int = 3) { for (int i = 0; i < 4; ++i) { min[i] = 0; max[i] = 0; } }
    };

    struct Direction { int x[3]; };

    template<class C, unsigned D>
    struct Point
    {
        C v[D];
        Point() { for (unsigned i = 0; i < D; ++i) v[i] = 0; }
        Point(const C* p) { for (unsigned i = 0; i < D; ++i) v[i] = p[i]; }
        C  operator[](unsigned i) const { return v[i]; }
    };

    struct BlockID { int gid; int proc; };

    namespace mpi
    {
        struct communicator
        {
            MPI_Comm comm;
            communicator(MPI_Comm c = MPI_COMM_WORLD): comm(c) {}
            operator MPI_Comm() const { return comm; }
            int rank() const { return 0; }
            int size() const { return 1; }
        };
    }

    struct MemoryBuffer
    {
        std::vector<char> buffer;
        size_t position = 0;
    };
    typedef MemoryBuffer BinaryBuffer;

    template<class T> struct Serialization;

    template<class T> inline void save(BinaryBuffer& bb, const T& x)
    {
        const char* p = reinterpret_cast<const char*>(&x);
        bb.buffer.insert(bb.buffer.end(), p, p + sizeof(T));
    }
    template<class T> inline void save(BinaryBuffer& bb, const T* x, size_t n)
    {
        const char* p = reinterpret_cast<const char*>(x);
        bb.buffer.insert(bb.buffer.end(), p, p + sizeof(T) * n);
    }
    template<class T> inline void load(BinaryBuffer& bb, T& x)
    {
        std::memcpy(&x, &bb.buffer[bb.position], sizeof(T));
        bb.position += sizeof(T);
    }
    template<class T> inline void load(BinaryBuffer& bb, T* x, size_t n)
    {
        if (n) std::memcpy(x, &bb.buffer[bb.position], sizeof(T) * n);
        bb.position += sizeof(T) * n;
    }

    struct Link
    {
        std::vector<BlockID> neighbors;
        virtual ~Link() {}
        int size() const { return (int)neighbors.size(); }
        BlockID target(int i) const { return neighbors[i]; }
    };

    struct RegularContinuousLink: public Link
    {
        std::vector<ContinuousBounds> cores;
        RegularContinuousLink() {}
        RegularContinuousLink(const RegularContinuousLink& o): Link(o), cores(o.cores) {}
        const ContinuousBounds& core(int i) const { return cores[i]; }
    };

    // neighbours whose core bounds contain p (inclusive on every face)
    template<class OutIter>
    void in(const RegularContinuousLink& link, const Point<float,3>& p, OutIter out,
            const ContinuousBounds&)
    {
        for (int n = 0; n < link.size(); ++n)
        {
            const ContinuousBounds& b = link.core(n);
            bool inside = true;
            for (int i = 0; i < 3; ++i)
                if (p[i] < b.min[i] || p[i] > b.max[i])
                    inside = false;
            if (inside)
                *out++ = n;
        }
    }

    struct Assigner
    {
        virtual ~Assigner() {}
        int rank(int) const { return 0; }
    };
    struct StaticAssigner: public Assigner {};
    struct RoundRobinAssigner: public StaticAssigner
    {
        RoundRobinAssigner(int = 1, int = -1) {}
    };

    struct Master
    {
        struct ProxyWithLink
        {
            Master* m;
            int     lid;
            Link*   link() const { return m->links_[lid]; }
            template<class T> void enqueue(const BlockID& to, const T& x) const
            {
                const char* p = reinterpret_cast<const char*>(&x);
                std::vector<char>& q = m->outgoing_[m->gids_[lid]][to.gid];
                q.insert(q.end(), p, p + sizeof(T));
            }
            void incoming(std::vector<int>& from) const
            {
                from.clear();
                for (auto& kv : m->incoming_[m->gids_[lid]])
                    from.push_back(kv.first);
            }
            MemoryBuffer& incoming(int from) const { return m->incoming_[m->gids_[lid]][from]; }
            template<class T> void dequeue(int from, T* x, size_t n) const
            {
                MemoryBuffer& mb = m->incoming_[m->gids_[lid]][from];
                if (n) std::memcpy(x, &mb.buffer[mb.position], sizeof(T) * n);
                mb.position += sizeof(T) * n;
            }
        };

        mpi::communicator                          comm_;
        std::vector<void*>                         blocks_;
        std::vector<Link*>                         links_;
        std::vector<int>                           gids_;
        std::map<int, std::map<int, std::vector<char> > >  outgoing_;  // from gid -> to gid -> bytes
        std::map<int, std::map<int, MemoryBuffer> >        incoming_;  // to gid -> from gid -> bytes

        Master() {}
        template<class... A> Master(A&&...) {}
        ~Master() { for (Link* l : links_) delete l; }

        void add(int gid, void* b, Link* l) { gids_.push_back(gid); blocks_.push_back(b); links_.push_back(l); }
        size_t size() const { return blocks_.size(); }
        template<class B> B* block(int i) const { return static_cast<B*>(blocks_[i]); }
        int lid(int gid) const
        {
            for (size_t i = 0; i < gids_.size(); ++i) if (gids_[i] == gid) return (int)i;
            return -1;
        }
        const mpi::communicator& communicator() const { return comm_; }

        template<class F> void foreach(const F& f)
        {
            for (size_t i = 0; i < blocks_.size(); ++i)
            {
                ProxyWithLink cp { this, (int)i };
                f(static_cast<typename first_arg<F>::type>(blocks_[i]), cp);
            }
        }
        void exchange()
        {
            incoming_.clear();
            for (auto& from : outgoing_)
                for (auto& to : from.second)
                {
                    MemoryBuffer& mb = incoming_[to.first][from.first];
                    mb.buffer = to.second;
                    mb.position = 0;
                }
            outgoing_.clear();
        }

        // deduce the block pointer type of a foreach callback
        template<class F> struct first_arg: first_arg<decltype(&F::operator())> {};
        template<class C, class R, class B, class P> struct first_arg<R (C::*)(B, P) const> { typedef B type; };
    };
}

#endif
