// The reference's C++ factories through include/sbgpu/compat.hpp, on the
// reference's own test inputs (test/test_block_integrate.cu:113-326 shapes).
// Prints the condensed / dense results, one value per line, for the caller to
// compare with the oracle.  Needs a GPU.
#include <sbgpu/compat.hpp>

#include <chrono>
#include <cstdio>

template <typename T>
static std::vector<sb::Pcf<T, T>> five()
{
  using P = sb::TimePoint<T, T>;
  std::vector<sb::Pcf<T, T>> v;
  v.emplace_back(std::vector<P>{{0, 1}, {1, 0}});
  v.emplace_back(std::vector<P>{{0, 2}, {T(0.5), 1}, {T(1.5), 0}});
  v.emplace_back(std::vector<P>{{0, 0}, {1, 3}, {2, 0}});
  v.emplace_back(std::vector<P>{{0, 5}});
  v.emplace_back(std::vector<P>{{0, 1}, {T(0.25), 2}, {T(0.75), 1}, {1, 0}});
  return v;
}

template <typename T>
static void run(const char* tag)
{
  auto pcfs = five<T>();
  sb::DistanceMatrix<T> dm(pcfs.size());
  auto t1 = sb::create_cuda_block_integrate_l1_task(dm, pcfs);
  t1->start_async(sb::default_executor());
  while (!t1->wait_for(std::chrono::milliseconds(10))) { }
  for (size_t k = 0; k < dm.storage_count(); ++k) std::printf("%s l1 %.17g\n", tag, (double)dm.data()[k]);

  sb::DistanceMatrix<T> d2(pcfs.size());
  auto t2 = sb::create_cuda_block_integrate_lp_task(d2, pcfs, T(2));
  t2->start_async(0);
  t2->wait();
  for (size_t k = 0; k < d2.storage_count(); ++k) std::printf("%s l2 %.17g\n", tag, (double)d2.data()[k]);

  sb::SymmetricMatrix<T> sm(pcfs.size());
  auto t3 = sb::create_cuda_block_integrate_l2_kernel_task(sm, pcfs);
  t3->start_async(0);
  t3->wait();
  for (size_t k = 0; k < sm.storage_count(); ++k) std::printf("%s k %.17g\n", tag, (double)sm.data()[k]);

  std::vector<sb::Pcf<T, T>> rows(pcfs.begin(), pcfs.begin() + 2), cols(pcfs.begin() + 2, pcfs.end());
  std::vector<T> dense(rows.size() * cols.size(), T(-1));
  auto t4 = sb::create_cuda_block_cdist_l1_task(dense.data(), rows, cols);
  t4->start_async(0);
  t4->wait();
  for (T v : dense) std::printf("%s c %.17g\n", tag, (double)v);

  bool rejected = false;
  try { sb::create_cuda_block_integrate_l1_task(dm, pcfs, T(1)); } catch (const std::invalid_argument&) { rejected = true; }
  std::printf("%s range_rejected %d\n", tag, rejected ? 1 : 0);
}

// The reference's known answers (test/test_l1_dist.cu:98-124): two
// default-constructed PCFs are at distance 0, and {(0,3),(1,0)} against
// {(0,1),(2,0)} at L1 distance 3, read back through operator() both ways.
template <typename T>
static void known_answers(const char* tag)
{
  using P = sb::TimePoint<T, T>;
  std::vector<sb::Pcf<T, T>> empty;
  empty.resize(2);
  sb::DistanceMatrix<T> d0(2);
  auto t0 = sb::create_cuda_block_integrate_l1_task(d0, empty);
  t0->start_async(0);
  t0->wait();
  std::printf("%s kat_empty %.17g\n", tag, (double)T(d0(0, 1)));

  std::vector<sb::Pcf<T, T>> two;
  two.emplace_back(std::vector<P>{{T(0), T(3)}, {T(1), T(0)}});
  two.emplace_back(std::vector<P>{{T(0), T(1)}, {T(2), T(0)}});
  sb::DistanceMatrix<T> d1(2);
  auto t1 = sb::create_cuda_block_integrate_l1_task(d1, two);
  t1->start_async(0);
  t1->wait();
  std::printf("%s kat_two %.17g %.17g %.17g %.17g\n", tag, (double)T(d1(0, 0)), (double)T(d1(0, 1)),
              (double)T(d1(1, 0)), (double)T(d1(1, 1)));
}

int main()
{
  run<float>("f32");
  run<double>("f64");
  known_answers<float>("f32");
  known_answers<double>("f64");
  return 0;
}
