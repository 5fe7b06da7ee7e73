/* Host build of the reference: the device-launch header carries nothing here.
 * Test infrastructure only (oracle pinning); never part of the product. */
#pragma once
