// vdb_mapping/OccupancyVDBMapping.hpp — drop-in for the reference's
// include/vdb_mapping/OccupancyVDBMapping.hpp (Config OccupancyVDBMapping.hpp:38-44,
// class :46-200), backed by libvdb_gb300.so. The log-odds constants are
// computed by the library on the host exactly as OccupancyVDBMapping.hpp:79-87
// does; the hit/miss node updates (:92-117) run in the GPU sweep kernel.
#ifndef VDB_MAPPING_GB300_OCCUPANCY_VDB_MAPPING_HPP
#define VDB_MAPPING_GB300_OCCUPANCY_VDB_MAPPING_HPP

#include "VDBMapping.hpp"

namespace vdb_mapping {

/*!
 * \brief Accumulation of configuration parameters (OccupancyVDBMapping.hpp:38-44).
 */
struct Config : BaseConfig
{
  double prob_hit       = 0.0;
  double prob_miss      = 0.0;
  double prob_thres_min = 0.0;
  double prob_thres_max = 0.0;
};

class OccupancyVDBMapping : public VDBMapping<float, Config>
{
public:
  explicit OccupancyVDBMapping(const double resolution)
    : VDBMapping<float, Config>(resolution)
  {
  }

  /*! OccupancyVDBMapping.hpp:59-89 over VDBMapping.hpp:1456-1469: same
   * messages and early returns. */
  inline void setConfig(const Config& config) override
  {
    vdbg_config c{};
    c.max_range           = config.max_range;
    c.fast_mode           = config.fast_mode ? 1 : 0;
    c.accumulation_period = config.accumulation_period;
    c.prob_hit            = config.prob_hit;
    c.prob_miss           = config.prob_miss;
    c.prob_thres_min      = config.prob_thres_min;
    c.prob_thres_max      = config.prob_thres_max;
    const int s           = vdbg_set_config(m_dev->map, &c);
    if (s == VDBG_ERR_BAD_RANGE)
    {
      std::cerr << "Max range of " << config.max_range << " invalid. Range cannot be negative." << std::endl;
      return;
    }
    m_config_set = true;
    if (s == VDBG_ERR_BAD_PROBABILITY)
    {
      if (config.prob_miss > 0.5)
        std::cerr << "Probability for a miss should be below 0.5 but is " << config.prob_miss << std::endl;
      else
        std::cerr << "Probability for a hit should be above 0.5 but is " << config.prob_hit << std::endl;
      return;
    }
    check(s, "vdbg_set_config");
  }
};

} // namespace vdb_mapping

#endif
