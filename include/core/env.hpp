// QTNH environment on one GB300: device selection and the stream all tensor operations
// of this environment are issued on. Replaces the reference's MPI environment
// (include/core/env.hpp:10-26, src/core/env.cpp:9-29): one process drives one GPU and
// holds every slab of every tensor, so proc_id is 0 and num_processes is 1.
#ifndef QTNH_CORE_ENV_HPP
#define QTNH_CORE_ENV_HPP

namespace qtnh {
  struct QTNHEnv {
    public:
      unsigned int proc_id;        ///< ID of the calling process (always 0).
      unsigned int num_processes;  ///< Number of processes (always 1).
      int device;                  ///< CUDA device the environment uses.
      void* stream;                ///< cudaStream_t of the environment (non-blocking).

      /// Selects device 0 (or $QTNH_DEVICE) and creates the environment's stream.
      /// Throws std::runtime_error when no GPU is visible.
      QTNHEnv();
      /// Synchronises and destroys the stream.
      ~QTNHEnv();
      QTNHEnv(const QTNHEnv&) = delete;
      QTNHEnv& operator=(const QTNHEnv&) = delete;

      /// Blocks until every operation issued on the environment's stream has finished.
      void synchronize() const;

      /// Prints environment information.
      void print() const;
  };
}

#endif
