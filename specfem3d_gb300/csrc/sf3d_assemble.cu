// Inter-slice assembly of the acceleration through MPI interface buffers.
//
// Entry points and semantics of assemble_MPI_vector_cuda.cu (the GPU side of
// assemble_MPI_vector.f90:243-384): the accel values of each interface's
// points are packed into buffer(NDIM, max_nibool, num_interfaces)
// (kernels/prepare_boundary_accel_on_device.cu), copied to the host for the
// MPI exchange, and the neighbours' contributions are added back into accel
// (kernels/assemble_boundary_accel_on_device.cu).  A point shared by several
// interfaces receives each contribution once per interface, as in the
// reference.  Packing and assembly run on the compute stream; the
// asynchronous variants copy through library-owned pinned buffers on a
// separate copy stream.
#include <string.h>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

// one thread per (point, interface); buffer layout (3, max_nibool, num_interfaces)
__global__ void pack_interfaces_kernel(const float* __restrict__ accel, float* __restrict__ buf, int num_interfaces,
                                       int max_nibool, const int* __restrict__ nibool, const int* __restrict__ ibool_if) {
  const long id = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (long)num_interfaces * max_nibool) return;
  const int iface = (int)(id / max_nibool);
  const int ip = (int)(id - (long)iface * max_nibool);
  if (ip >= nibool[iface]) return;
  const int g = ibool_if[id];
  buf[3 * id] = accel[3L * g];
  buf[3 * id + 1] = accel[3L * g + 1];
  buf[3 * id + 2] = accel[3L * g + 2];
}

__global__ void assemble_interfaces_kernel(float* __restrict__ accel, const float* __restrict__ buf,
                                           int num_interfaces, int max_nibool, const int* __restrict__ nibool,
                                           const int* __restrict__ ibool_if) {
  const long id = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (long)num_interfaces * max_nibool) return;
  const int iface = (int)(id / max_nibool);
  const int ip = (int)(id - (long)iface * max_nibool);
  if (ip >= nibool[iface]) return;
  const int g = ibool_if[id];
  atomicAdd(accel + 3L * g, buf[3 * id]);
  atomicAdd(accel + 3L * g + 1, buf[3 * id + 1]);
  atomicAdd(accel + 3L * g + 2, buf[3 * id + 2]);
}

float* pick_accel(Mesh* mp, int fa) { return fa == 3 ? mp->b.accel : mp->f.accel; }
float* pick_buffer(Mesh* mp, int fa) { return fa == 3 ? mp->d_b_send_accel_buffer : mp->d_send_accel_buffer; }

void pack(Mesh* mp, int fa) {
  const long n = (long)mp->num_interfaces * mp->max_nibool_interfaces;
  pack_interfaces_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(pick_accel(mp, fa), pick_buffer(mp, fa),
                                                               mp->num_interfaces, mp->max_nibool_interfaces,
                                                               mp->d_nibool_interfaces, mp->d_ibool_interfaces);
}

void assemble(Mesh* mp, int fa) {
  const long n = (long)mp->num_interfaces * mp->max_nibool_interfaces;
  assemble_interfaces_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(pick_accel(mp, fa), pick_buffer(mp, fa),
                                                                   mp->num_interfaces, mp->max_nibool_interfaces,
                                                                   mp->d_nibool_interfaces, mp->d_ibool_interfaces);
}

bool interfaces_match(Mesh* mp, const int* num_interfaces, const int* max_nibool) {
  if ((num_interfaces && *num_interfaces != mp->num_interfaces) ||
      (max_nibool && *max_nibool != mp->max_nibool_interfaces))
    return set_error(SF3D_ERR_ARG, "interface sizes differ from prepare_constants_device");
  return true;
}

bool check_fa(Mesh* mp, const int* fa) {
  if (!fa || (*fa != 1 && *fa != 3)) return set_error(SF3D_ERR_ARG, "FORWARD_OR_ADJOINT must be 1 or 3");
  if (!pick_accel(mp, *fa)) return set_error(SF3D_ERR_STATE, "field not allocated");
  return true;
}

}  // namespace

bool prepare_interfaces(Mesh* mp, int num_interfaces, int max_nibool, const int* nibool, const int* ibool_if) {
  if (num_interfaces <= 0) return true;
  if (max_nibool <= 0 || !nibool || !ibool_if) return set_error(SF3D_ERR_ARG, "invalid MPI interface arrays");
  std::vector<int> ib((size_t)num_interfaces * max_nibool, 0);
  for (int i = 0; i < num_interfaces; ++i) {
    if (nibool[i] < 0 || nibool[i] > max_nibool) return set_error(SF3D_ERR_ARG, "nibool_interfaces exceeds max_nibool");
    for (int p = 0; p < nibool[i]; ++p) {
      const int g = ibool_if[p + (long)max_nibool * i];
      if (g < 1 || g > mp->nglob) return set_error(SF3D_ERR_ARG, "ibool_interfaces entry out of range [1, NGLOB_AB]");
      ib[p + (size_t)max_nibool * i] = g - 1;
    }
  }
  mp->num_interfaces = num_interfaces;
  mp->max_nibool_interfaces = max_nibool;
  mp->size_mpi_buffer = 3L * max_nibool * num_interfaces;
  const size_t bytes = sizeof(float) * mp->size_mpi_buffer;
  bool ok = cuda_ok(cudaStreamCreateWithFlags(&mp->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate") &&
            cuda_ok(cudaEventCreateWithFlags(&mp->ev_pack, cudaEventDisableTiming), "cudaEventCreate") &&
            alloc_zero((void**)&mp->d_nibool_interfaces, sizeof(int) * num_interfaces) &&
            alloc_zero((void**)&mp->d_ibool_interfaces, sizeof(int) * ib.size()) &&
            alloc_zero((void**)&mp->d_send_accel_buffer, bytes) &&
            alloc_zero((void**)&mp->d_b_send_accel_buffer, bytes) &&
            cuda_ok(cudaMallocHost((void**)&mp->h_send_accel_buffer, bytes), "cudaMallocHost") &&
            cuda_ok(cudaMallocHost((void**)&mp->h_recv_accel_buffer, bytes), "cudaMallocHost");
  ok = ok && copy_sync(mp->d_nibool_interfaces, nibool, sizeof(int) * num_interfaces, cudaMemcpyHostToDevice, mp->stream) &&
       copy_sync(mp->d_ibool_interfaces, ib.data(), sizeof(int) * ib.size(), cudaMemcpyHostToDevice, mp->stream);
  return ok;
}

void free_interfaces(Mesh* mp) {
  cudaFree(mp->d_nibool_interfaces); cudaFree(mp->d_ibool_interfaces);
  cudaFree(mp->d_send_accel_buffer); cudaFree(mp->d_b_send_accel_buffer);
  if (mp->h_send_accel_buffer) cudaFreeHost(mp->h_send_accel_buffer);
  if (mp->h_recv_accel_buffer) cudaFreeHost(mp->h_recv_accel_buffer);
  if (mp->copy_stream) cudaStreamDestroy(mp->copy_stream);
  if (mp->ev_pack) cudaEventDestroy(mp->ev_pack);
  mp->num_interfaces = 0;
  mp->size_mpi_buffer = 0;
}

}  // namespace sf3d

using namespace sf3d;

extern "C" {

void transfer_boun_accel_from_device_(long* Mesh_pointer, realw* send_accel_buffer, const int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || mp->size_mpi_buffer == 0) return;
  if (!check_fa(mp, FORWARD_OR_ADJOINT)) return;
  pack(mp, *FORWARD_OR_ADJOINT);
  if (!cuda_ok(cudaGetLastError(), "pack_interfaces_kernel")) return;
  copy_sync(send_accel_buffer, pick_buffer(mp, *FORWARD_OR_ADJOINT), sizeof(float) * mp->size_mpi_buffer,
            cudaMemcpyDeviceToHost, mp->stream);
}

void transfer_boundary_from_device_a_(long* Mesh_pointer, const int* nspec_outer_elastic) {
  (void)nspec_outer_elastic;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || mp->size_mpi_buffer == 0) return;
  pack(mp, 1);
  if (!cuda_ok(cudaGetLastError(), "pack_interfaces_kernel")) return;
  // the copy stream waits for the packing kernel, then copies while compute continues
  if (!cuda_ok(cudaEventRecord(mp->ev_pack, mp->stream), "cudaEventRecord")) return;
  if (!cuda_ok(cudaStreamWaitEvent(mp->copy_stream, mp->ev_pack, 0), "cudaStreamWaitEvent")) return;
  cuda_ok(cudaMemcpyAsync(mp->h_send_accel_buffer, mp->d_send_accel_buffer, sizeof(float) * mp->size_mpi_buffer,
                          cudaMemcpyDeviceToHost, mp->copy_stream),
          "cudaMemcpyAsync");
}

void sync_copy_from_device_(long* Mesh_pointer, int* iphase, realw* send_buffer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!iphase || *iphase != 2) { set_error(SF3D_ERR_ARG, "sync_copy_from_device must be called for iphase == 2"); return; }
  if (mp->size_mpi_buffer == 0) return;
  if (!cuda_ok(cudaStreamSynchronize(mp->copy_stream), "cudaStreamSynchronize")) return;
  memcpy(send_buffer, mp->h_send_accel_buffer, sizeof(float) * mp->size_mpi_buffer);
}

void transfer_boundary_to_device_a_(long* Mesh_pointer, realw* buffer_recv_vector_ext_mesh,
                                    const int* num_interfaces_ext_mesh, const int* max_nibool_interfaces_ext_mesh) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || mp->size_mpi_buffer == 0) return;
  if (!interfaces_match(mp, num_interfaces_ext_mesh, max_nibool_interfaces_ext_mesh)) return;
  // the previous asynchronous download of the send buffer must be complete before
  // the buffer is overwritten
  if (!cuda_ok(cudaStreamSynchronize(mp->copy_stream), "cudaStreamSynchronize")) return;
  memcpy(mp->h_recv_accel_buffer, buffer_recv_vector_ext_mesh, sizeof(float) * mp->size_mpi_buffer);
  cuda_ok(cudaMemcpyAsync(mp->d_send_accel_buffer, mp->h_recv_accel_buffer, sizeof(float) * mp->size_mpi_buffer,
                          cudaMemcpyHostToDevice, mp->copy_stream),
          "cudaMemcpyAsync");
}

void transfer_asmbl_accel_to_device_(long* Mesh_pointer, realw* buffer_recv_vector_ext_mesh,
                                     const int* num_interfaces_ext_mesh, const int* max_nibool_interfaces_ext_mesh,
                                     const int* nibool_interfaces_ext_mesh, const int* ibool_interfaces_ext_mesh,
                                     const int* FORWARD_OR_ADJOINT) {
  (void)nibool_interfaces_ext_mesh; (void)ibool_interfaces_ext_mesh;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || mp->size_mpi_buffer == 0) return;
  if (!interfaces_match(mp, num_interfaces_ext_mesh, max_nibool_interfaces_ext_mesh)) return;
  if (!check_fa(mp, FORWARD_OR_ADJOINT)) return;
  const int fa = *FORWARD_OR_ADJOINT;
  if (!copy_sync(pick_buffer(mp, fa), buffer_recv_vector_ext_mesh, sizeof(float) * mp->size_mpi_buffer,
                 cudaMemcpyHostToDevice, mp->stream))
    return;
  assemble(mp, fa);
  cuda_ok(cudaGetLastError(), "assemble_interfaces_kernel");
}

void transfer_sync_accel_to_device_(long* Mesh_pointer, realw* buffer_recv_vector_ext_mesh,
                                    const int* num_interfaces_ext_mesh, const int* max_nibool_interfaces_ext_mesh,
                                    const int* nibool_interfaces_ext_mesh, const int* ibool_interfaces_ext_mesh,
                                    const int* FORWARD_OR_ADJOINT) {
  (void)nibool_interfaces_ext_mesh; (void)ibool_interfaces_ext_mesh;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || mp->size_mpi_buffer == 0) return;
  if (!interfaces_match(mp, num_interfaces_ext_mesh, max_nibool_interfaces_ext_mesh)) return;
  if (!check_fa(mp, FORWARD_OR_ADJOINT)) return;
  const int fa = *FORWARD_OR_ADJOINT;
  if (fa == 1) {
    // the receive buffer was uploaded by transfer_boundary_to_device_a on the copy stream
    if (!cuda_ok(cudaStreamSynchronize(mp->copy_stream), "cudaStreamSynchronize")) return;
  } else {
    if (!copy_sync(pick_buffer(mp, fa), buffer_recv_vector_ext_mesh, sizeof(float) * mp->size_mpi_buffer,
                   cudaMemcpyHostToDevice, mp->stream))
      return;
  }
  assemble(mp, fa);
  cuda_ok(cudaGetLastError(), "assemble_interfaces_kernel");
}

}  // extern "C"
