// Empty stand-in: nothing of it is used by the host calculators.
#pragma once
