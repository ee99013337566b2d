set output "hist_group1_MOTIF00005.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-50.0689:11.6327]
set yrange [0:133658]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00005.dat" using 1:2 title 'MOTIF00005 (group1)' with boxes
