// Kinematic-bicycle-on-costmap and dynamic-bicycle (slip) instantiations of the engine.
#include "mg_engine.cuh"

namespace mg
{
mppi_status create_bicycle_costmap_engine(const CreateArgs& a, EngineBase** out)
{
  return Engine<BicycleCostmapModel>::create(a, out);
}

mppi_status create_bicycle_slip_engine(const CreateArgs& a, EngineBase** out)
{
  return Engine<BicycleSlipModel>::create(a, out);
}
}  // namespace mg

namespace mg
{
mppi_status create_bicycle_slip_mlp_engine(const CreateArgs& a, EngineBase** out)
{
  return Engine<BicycleSlipMLPModel>::create(a, out);
}
}  // namespace mg
